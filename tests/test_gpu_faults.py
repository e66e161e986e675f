"""Failure paths of the GPU Newton path, driven from the host (no GPU fault):

- a sync-free ILU(0) sweep whose dependency wait runs out (a reversed node
  order on one CTA, with a short wait limit set through gb_set_sweep_fault):
  the linear solve returns -1 with its message, and the same context then
  solves the same system exactly as before;
- a NaN in the Newton state: gb_solve_nonlinear_problem returns -1 on the
  non-finite residual norm (the reference's check,
  src/mm_sol_nonlinear.c:1487-1491), and the context solves the next
  problem normally;
- a Krylov limit too small to converge: Newton reports "not converged"
  (return 0, converged 0) and a normal solve from the state it left
  converges to the oracle's solution.
"""
import numpy as np
import pytest

import oracle
from goma_gb300 import _lib
from goma_gb300 import problem as pb
from goma_gb300.newton import GomaNewton

pytestmark = pytest.mark.gpu


def _scaled_system(prob, seed):
    o = oracle.Oracle(prob)
    x = o.dirichlet_init(np.random.default_rng(seed).uniform(-0.5, 0.5, o.N))
    R, a, st = o.matrix_fill(x)
    assert st == 0
    a_s, R_s, _ = o.row_sum_scale(a, R)
    return o, a_s, R_s


@pytest.mark.parametrize("prob_fn", [lambda: pb.boussinesq_cube_3d(3, 1e4, 0.71),
                                     lambda: pb.lid_cavity_2d(8, 100.0)],
                         ids=["cube", "cavity"])
@pytest.mark.parametrize("fp32", [False, True], ids=["fp64", "fp32_refined"])
def test_sweep_wait_gives_up_and_the_context_recovers(fp32, prob_fn):
    """Both sync-free sweep kernels: a CTA per node (the HEX27 cube's long
    rows, and the cavity's FP64 sweeps) and a warp per node (the QUAD9
    cavity's FP32 sweeps: short rows)."""
    prob = prob_fn()
    o, a_s, R_s = _scaled_system(prob, 2)
    gn = GomaNewton(prob)
    gn.set_triangular_solve(0)   # the sync-free sweeps
    opts = dict(linear_tol=1e-10, max_linear_its=300, krylov_dim=60, fp32_inner=fp32)
    dx_ref, its_ref, rr_ref = gn.linear_solve(a_s, R_s, **opts)
    assert rr_ref <= 1e-10
    gn.set_sweep_fault(spin_limit=10000, reverse_lower=True)
    with pytest.raises(_lib.GbError, match="dependency wait gave up"):
        # every later wait of the failed solve stops within 1024 polls; a few
        # iterations and one refinement keep that short
        gn.linear_solve(a_s, R_s, **dict(opts, max_linear_its=3, max_refinements=1))
    gn.set_sweep_fault()
    dx, its, rr = gn.linear_solve(a_s, R_s, **opts)
    assert its == its_ref
    assert np.array_equal(dx, dx_ref)   # the sweeps and GMRES are deterministic


def test_nan_state_returns_an_error_and_the_context_recovers():
    prob = pb.lid_cavity_2d(6, 100.0)
    o = oracle.Oracle(prob)
    xo, it, _ = o.newton(o.dirichlet_init(np.zeros(o.N)), 30, 1e-11)
    assert it > 0
    gn = GomaNewton(prob)
    x0 = gn.dirichlet_init(np.zeros(gn.N))
    free = np.flatnonzero(~o.dirichlet_mask())
    x_bad = x0.copy()
    x_bad[free[len(free) // 2]] = np.nan
    with pytest.raises(_lib.GbError, match="non-finite residual norm"):
        gn.solve_nonlinear_problem(x_bad, residual_tol=1e-11, linear_tol=1e-10)
    x, conv, st = gn.solve_nonlinear_problem(x0, residual_tol=1e-11, linear_tol=1e-10)
    assert conv
    assert np.abs(x - xo).max() <= 1e-8 * np.abs(xo).max()


def test_krylov_limit_reports_not_converged_without_corrupting_state():
    prob = pb.lid_cavity_2d(6, 100.0)
    o = oracle.Oracle(prob)
    xo, it, _ = o.newton(o.dirichlet_init(np.zeros(o.N)), 30, 1e-11)
    gn = GomaNewton(prob)
    x1, conv, st = gn.solve_nonlinear_problem(None, residual_tol=1e-11, linear_tol=1e-10,
                                              max_linear_its=1, max_newton=3)
    assert not conv
    assert st["newton_its"] == 3 and st["linear_its"] <= 3
    assert np.isfinite(x1).all()
    x, conv, st = gn.solve_nonlinear_problem(x1, residual_tol=1e-11, linear_tol=1e-10,
                                             max_newton=40)
    assert conv
    assert np.abs(x - xo).max() <= 1e-8 * np.abs(xo).max()
