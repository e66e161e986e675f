"""Pseudo-arclength continuation (goma_gb300/arclength.py) on the CPU: the
1-D Bratu problem -u'' = lam exp(u), u(0) = u(1) = 0, whose solution
branch turns back at lam_c = 3.51383 (max u = 1.187 there).  Parameter
continuation stops at the fold; the arc-length driver goes round it onto
the upper branch.  Also the host row scaling of the library adapter
against the oracle's restatement of row_sum_scale_MSR."""
import numpy as np
import pytest

import oracle
from goma_gb300 import problem as pb
from goma_gb300.arclength import arclength_continuation, msr_row_scale

LAM_C = 3.513830719125162


class Bratu:
    def __init__(self, n=200):
        self.n = n
        self.h = 1.0 / (n + 1)

    def residual(self, u, lam):
        up = np.concatenate([[0.0], u, [0.0]])
        return (2.0 * u - up[:-2] - up[2:]) / self.h ** 2 - lam * np.exp(u)

    def linearize(self, u, lam):
        n, h2 = self.n, self.h ** 2
        J = (np.diag(np.full(n, 2.0 / h2) - lam * np.exp(u))
             + np.diag(np.full(n - 1, -1.0 / h2), 1) + np.diag(np.full(n - 1, -1.0 / h2), -1))
        return self.residual(u, lam), lambda rhs: np.linalg.solve(J, rhs), np.ones(n)


def _lower_branch(p, lam):
    u = np.zeros(p.n)
    for _ in range(30):
        R, solve, _ = p.linearize(u, lam)
        u = u + solve(-R)
    return u


def test_bratu_branch_goes_round_the_fold():
    p = Bratu()
    u1 = _lower_branch(p, 1.0)
    recs, sols = arclength_continuation(p, u1, 1.0, 0.2, 400, lam_bounds=(0.5, 4.0), tol=1e-9)
    lams = np.array([r["lam"] for r in recs])
    umax = np.array([s.max() for s in sols])
    assert all(r["residual"] < 1e-9 for r in recs[1:])
    # up the lower branch, round the fold, down the upper branch; the largest
    # sampled lam is near the fold and never beyond it
    k = int(np.argmax(lams))
    assert LAM_C - 0.01 < lams[k] <= LAM_C
    assert 0.9 < umax[k] < 1.5
    assert np.all(np.diff(umax) > 0)          # the branch is monotone in max u
    assert lams[-1] < 1.0 and umax[-1] > 3.0  # well onto the upper branch
    lamdot = np.array([r["lamdot"] for r in recs])
    assert lamdot[0] > 0 and lamdot[-1] < 0   # the tangent turned
    # a point on the upper branch is a solution that parameter continuation
    # from the lower branch does not reach
    j = len(recs) - 1
    assert np.abs(p.residual(sols[j], lams[j])).max() < 1e-6


def test_fine_steps_locate_the_fold():
    """Short steps from lam = 3.4 find the turning point of the 200-point
    discretisation within 1e-4 of the continuous problem's lam_c."""
    p = Bratu()
    recs, _ = arclength_continuation(p, _lower_branch(p, 3.4), 3.4, 0.005, 400,
                                     lam_bounds=(3.3, 4.0), tol=1e-9, ds_max=0.005)
    lams = np.array([r["lam"] for r in recs])
    assert abs(lams.max() - LAM_C) < 1e-4
    assert lams[-1] < 3.3  # turned and came back down


def test_direction_and_step_limits():
    p = Bratu(50)
    recs, _ = arclength_continuation(p, np.zeros(p.n), 0.0, 0.1, 5, direction=-1.0)
    lams = [r["lam"] for r in recs]
    assert lams[-1] < lams[0]
    with pytest.raises(RuntimeError, match="ds_min"):
        arclength_continuation(p, np.zeros(p.n), 0.0, 0.1, 3, max_corrector=1, ds_min=0.05)


@pytest.mark.parametrize("prob_fn", [lambda: pb.lid_cavity_2d(3),
                                     lambda: pb.boussinesq_cube_3d(2, 1e4, 0.71)],
                         ids=["cavity2d", "bouss3d"])
def test_host_row_scaling_matches_the_oracle(prob_fn):
    prob = prob_fn()
    o = oracle.Oracle(prob)
    x = o.dirichlet_init(np.random.default_rng(2).uniform(-1, 1, o.N))
    R, a, st = o.matrix_fill(x)
    a_ref, R_ref, s_ref = o.row_sum_scale(a, R)
    a_s, s = msr_row_scale(o.ija(), a)
    assert np.allclose(s, s_ref, rtol=1e-14, atol=0)
    ija = o.ija()
    used = np.r_[np.arange(o.N), np.arange(ija[0], ija[o.N])]
    assert np.allclose(a_s[used], a_ref[used], rtol=1e-14, atol=1e-300)
