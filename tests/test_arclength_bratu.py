"""Pseudo-arclength continuation of a Q2/P1 problem round a turning point:
the Frank-Kamenetskii / Bratu problem on the unit square (energy equation
with the heat source lam exp(T), T = 0 on the boundary, fluid at rest; its
heat-source assembly is pinned to the reference's in tests/golden/
bratu2d_*), whose solution branch folds at lam ~ 6.808.

The CPU run uses the oracle (direct solves) through the same driver
(goma_gb300.arclength); the GPU run keeps every vector on the device
(GomaArcProblemDevice: device assembly, row scaling and ILU(0)-GMRES) and
must follow the same path."""
import numpy as np
import pytest

import oracle
from goma_gb300 import arclength as arc
from goma_gb300 import problem as pb

N_EL = 8
LAM0, DS, STEPS = 1.0, 0.5, 26
FOLD_2D = 6.80812  # the continuous problem's fold (Bratu, unit square)


class OracleArcProblem:
    """linearize() from the CPU oracle: assembly, row-sum scaling, a sparse
    direct solve."""

    def __init__(self, n):
        self.n = n
        self._cache = {}

    def _oracle(self, lam):
        o = self._cache.get(lam)
        if o is None:
            o = oracle.Oracle(pb.bratu_square_2d(self.n, lam))
            self._cache = {lam: o}
        return o

    def residual(self, x, lam):
        R, _, st = self._oracle(lam).matrix_fill(x, jacobian=False)
        assert st == 0
        return R

    def linearize(self, x, lam):
        sp = pytest.importorskip("scipy.sparse")
        spl = pytest.importorskip("scipy.sparse.linalg")
        o = self._oracle(lam)
        R, a, st = o.matrix_fill(x)
        assert st == 0
        a_s, R_s, s = o.row_sum_scale(a, R)
        ija = o.ija()
        N = o.N
        rows = np.concatenate([np.arange(N), np.repeat(np.arange(N), np.diff(ija[:N + 1]))])
        cols = np.concatenate([np.arange(N), ija[N + 1:ija[N]]])
        vals = np.concatenate([a_s[:N], a_s[N + 1:ija[N]]])
        lu = spl.splu(sp.csc_matrix((vals, (rows, cols)), shape=(N, N)))
        return R_s, lu.solve, s


def _start(n):
    o = oracle.Oracle(pb.bratu_square_2d(n, LAM0))
    x, it, _ = o.newton(o.dirichlet_init(np.zeros(o.N)), 30, 1e-12)
    assert it > 0
    return x, o


def _fold(records):
    lam = np.array([r["lam"] for r in records])
    k = int(np.argmax(lam))
    assert 0 < k < len(lam) - 1, "the path must pass the fold"
    return lam, k


def test_oracle_arclength_passes_the_bratu_fold():
    x0, o = _start(N_EL)
    recs, sols = arc.arclength_continuation(OracleArcProblem(N_EL), x0, LAM0, DS, STEPS,
                                            tol=1e-10, ds_max=DS)
    lam, k = _fold(recs)
    assert abs(lam[k] - FOLD_2D) < 2e-2
    # past the fold lam falls again and the temperature keeps rising
    tmax = [float(np.max(np.abs(s))) for s in sols]
    assert lam[-1] < lam[k] - 0.5 and tmax[-1] > tmax[k] > tmax[0]


@pytest.mark.gpu
def test_gpu_arclength_follows_the_oracle_path_round_the_fold():
    import torch
    from goma_gb300.newton import GomaNewton
    x0, o = _start(N_EL)
    ref_recs, ref_sols = arc.arclength_continuation(OracleArcProblem(N_EL), x0, LAM0, DS,
                                                    STEPS, tol=1e-10, ds_max=DS)
    gn = GomaNewton(pb.bratu_square_2d(N_EL, LAM0))

    def set_lam(g, lam):
        m = g.problem.material
        m.heat_source = (lam, 1.0)
        g.set_material(m)

    prob = arc.GomaArcProblemDevice(gn, set_lam, linear_tol=1e-12, max_linear_its=2000)
    xd = torch.tensor(x0, dtype=torch.float64, device="cuda")
    recs, sols = arc.arclength_continuation(prob, xd, LAM0, DS, STEPS, tol=1e-10, ds_max=DS)
    assert len(recs) == len(ref_recs)
    lam = np.array([r["lam"] for r in recs])
    lam_ref = np.array([r["lam"] for r in ref_recs])
    assert np.abs(lam - lam_ref).max() <= 1e-7 * np.abs(lam_ref).max()
    for s, sr in zip(sols, ref_sols):
        s = s.cpu().numpy()
        assert np.abs(s - sr).max() <= 1e-7 * max(np.abs(sr).max(), 1e-30)
    _, k = _fold(recs)
    # every point of the device path solves the problem at its lam (oracle)
    for r, s in zip(recs, sols):
        R, _, st = oracle.Oracle(pb.bratu_square_2d(N_EL, r["lam"])).matrix_fill(
            s.cpu().numpy(), jacobian=False)
        assert st == 0 and np.abs(R).max() <= 1e-8
