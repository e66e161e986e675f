"""Analytic Jacobian against finite differences of the residual, the check
the reference's numerical_jacobian performs (src/mm_numjac.c:716): columns
perturbed by dx = 1e-7 |x| + 1e-10 (calc_numerical_delta, :1568), here as
central differences of the GPU residual along random directions, so the
whole matrix is exercised at once: J v ~ (R(x + h v) - R(x - h v)) / 2h."""
import numpy as np
import pytest

from goma_gb300 import problem as pb
from goma_gb300.newton import GomaNewton

pytestmark = pytest.mark.gpu


def msr_matvec(ija, a, v):
    N = ija[0] - 1
    y = a[:N] * v
    for i in range(N):
        lo, hi = ija[i], ija[i + 1]
        y[i] += np.dot(a[lo:hi], v[ija[lo:hi]])
    return y


@pytest.mark.parametrize("prob_fn", [
    lambda: pb.lid_cavity_2d(5, 100.0, mesh=pb.box_mesh(2, 5, 4, 1, 1.2, 1.0, amp=0.12, seed=2)),
    lambda: pb.carreau_step_2d(6, 3, 40.0, mesh=pb.box_mesh(2, 6, 3, 1, 3.0, 1.0, amp=0.1,
                                                            seed=4)),
    lambda: pb.boussinesq_cube_3d(2, 1e4, 0.71, mesh=pb.box_mesh(3, 2, 2, 2, amp=0.1, seed=6)),
], ids=["cavity2d", "carreau2d", "bouss3d"])
def test_analytic_jacobian_matches_finite_differences(prob_fn):
    prob = prob_fn()
    gn = GomaNewton(prob)
    rng = np.random.default_rng(3)
    x = gn.dirichlet_init(rng.uniform(-0.5, 0.5, gn.N))
    R0, a = gn.matrix_fill_full(x)
    ija = gn.msr_pattern()
    for trial in range(3):
        v = rng.uniform(-1, 1, gn.N)
        h = 1e-6
        Rp, _ = gn.matrix_fill_full(x + h * v, jacobian=False)
        Rm, _ = gn.matrix_fill_full(x - h * v, jacobian=False)
        fd = (Rp - Rm) / (2 * h)
        Jv = msr_matvec(ija, a, v)
        # Dirichlet rows hold R = 0 and an identity row: compare the others
        mask = np.abs(R0) > 0
        err = np.abs(Jv - fd)[mask].max() / np.abs(Jv[mask]).max()
        assert err < 1e-6, err


@pytest.mark.parametrize("name", ["cav2d_2x2", "cav2d_3x2_pert", "bfs2d_4x2_carreau",
                                  "box3d_2x2x2_bouss", "box3d_2x1x3_carreau_t",
                                  "box3d_2x2x2_species", "bratu2d_4x4_pert",
                                  "channel2d_4x3_ibc", "box3d_2x2x2_ibc"])
def test_gpu_jacobian_passes_the_reference_checker_like_the_reference(name):
    """The reference's own Jacobian checker (numerical_jacobian with
    Debug = -2, src/mm_numjac.c:716, restated in tests/numjac_check.py) on
    the GPU's assembly: every column of every golden assembly problem,
    perturbed around the golden state, flags exactly what the reference
    flagged when it checked its own analytic Jacobian on the same problem
    and state (tests/golden/numjac_reference.json, from running the
    reference; nothing)."""
    import json
    import os

    from tests import golden_cases as gc
    from tests import numjac_check as nj
    with open(os.path.join(gc.GOLDEN, "numjac_reference.json")) as f:
        ref = json.load(f)[name]
    g, case = gc.load(name)
    prob = nj.without_dirichlet(gc.problem_from_case(case))
    gn = GomaNewton(prob)
    assert gn.N == ref["columns"]
    ija = gn.msr_pattern()

    def fill(x):
        R, a = gn.matrix_fill_full(x)
        return R, nj.msr_to_dense(ija, a)

    fu = np.empty(prob.mesh.num_nodes + 1, np.int32)
    import ctypes

    from goma_gb300 import _lib
    _lib.check(gn._L.gb_first_unknown(gn.h, fu.ctypes.data_as(ctypes.POINTER(ctypes.c_int))))
    flagged = nj.check(nj.Layout(prob, fu), fill, g["x"])
    assert len(flagged) == len(ref["flagged"]), flagged[:5]
