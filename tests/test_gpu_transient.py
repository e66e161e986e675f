"""The transient path on the GPU: assembly with the time-derivative terms and
the reference's fixed-step time loop, against the reference's own transient
assemblies and runs (tests/golden/, made by running the reference) and
against the oracle's transient loop on a larger mesh.

- assembly: residual and Jacobian entries within 1e-12 (row-scaled) of the
  reference's first assembly of a time step at a seeded state and time
  derivative (mass terms of momentum, energy and species; both 3-D kernels);
- time loop: the solution after every step within 1e-8 of the reference's
  (three backward-Euler steps, then Crank-Nicolson with its second-order
  predictor), with FP64, FP32-refined and FP32-preconditioner linear solves.
"""
import numpy as np
import pytest

import oracle
from goma_gb300 import problem as pb
from goma_gb300.newton import GomaNewton
from tests import golden_cases as gc

pytestmark = pytest.mark.gpu
TOL = 1e-12
TOL_X = 1e-8


@pytest.mark.parametrize("path", [0, 1], ids=["automatic", "scalar"])
@pytest.mark.parametrize("name", gc.names("assemble", transient=True))
def test_gpu_transient_assembly_matches_reference(name, path):
    g, case = gc.load(name)
    gn = GomaNewton(gc.problem_from_case(case))
    gn.set_assembly_path(path)
    assert np.array_equal(gn.msr_pattern(), g["ija"])
    dt, theta = g["delta_t_theta"]
    R, a = gn.matrix_fill_full_transient(g["x"], g["xdot"], dt, theta)
    assert gc.msr_row_scaled_error(g["ija"], a, g["a"]) < TOL
    assert np.abs(R - g["R"]).max() <= TOL * np.abs(g["R"]).max()
    # residual-only fill gives the same residual
    R2, _ = gn.matrix_fill_full_transient(g["x"], g["xdot"], dt, theta, jacobian=False)
    assert np.abs(R2 - g["R"]).max() <= TOL * np.abs(g["R"]).max()


PRECISIONS = {"fp64": {}, "fp32_refined": {"fp32_inner": True},
              "fp32_preconditioner": {"fp32_preconditioner": True}}


@pytest.mark.parametrize("precision", list(PRECISIONS))
@pytest.mark.parametrize("name", gc.names("transient"))
def test_gpu_time_loop_matches_reference(name, precision):
    g, case = gc.load(name)
    tr = case["transient"]
    gn = GomaNewton(gc.problem_from_case(case))
    xs, st = gn.solve_transient(tr["steps"], tr["dt"], tr["theta"], residual_tol=case["tol"],
                                linear_tol=1e-13, max_linear_its=3000, krylov_dim=60,
                                max_newton=30, **PRECISIONS[precision])
    assert st["steps_done"] == tr["steps"]
    ref = g["x_steps"]
    for k in range(tr["steps"]):
        assert np.abs(xs[k] - ref[k]).max() <= TOL_X * np.abs(ref[k]).max(), k


def test_gpu_time_loop_matches_oracle_on_a_larger_cavity():
    """16 x 16 lid-driven cavity at Re 100, six steps of 0.02 from rest."""
    prob = pb.lid_cavity_2d(16, 100.0)
    o = oracle.Oracle(prob)
    ref = o.transient_run(np.zeros(o.N), 6, 0.02, 0.5, tol=1e-11)
    gn = GomaNewton(prob)
    xs, st = gn.solve_transient(6, 0.02, 0.5, residual_tol=1e-11, linear_tol=1e-12,
                                max_linear_its=3000, krylov_dim=60)
    for k in range(6):
        assert np.abs(xs[k] - ref[k]).max() <= TOL_X * np.abs(ref[k]).max(), k


def test_gpu_transient_step_matches_the_time_loop():
    """One step through gb_solve_nonlinear_problem_transient from the
    backward-Euler prediction (x_old, xdot = 0) equals the first step of the
    time loop."""
    g, case = gc.load("cav2d_8x8_transient")
    tr = case["transient"]
    gn = GomaNewton(gc.problem_from_case(case))
    x0 = gn.dirichlet_init(np.zeros(gn.N))
    x, xd, conv, st = gn.solve_transient_step(x0, np.zeros(gn.N), tr["dt"], 0.0,
                                              residual_tol=1e-12, linear_tol=1e-13,
                                              max_linear_its=3000, krylov_dim=60)
    assert conv
    ref = g["x_steps"][0]
    assert np.abs(x - ref).max() <= TOL_X * np.abs(ref).max()
    # xdot followed every update: it is (x - x_old) / dt for backward Euler
    assert np.abs(xd - (x - x0) / tr["dt"]).max() <= 1e-9 * np.abs(xd).max()


def test_gpu_transient_rejects_bad_steps():
    from goma_gb300 import _lib
    gn = GomaNewton(pb.lid_cavity_2d(2, 10.0))
    x = np.zeros(gn.N)
    with pytest.raises(_lib.GbError, match="delta_t must be positive"):
        gn.matrix_fill_full_transient(x, x, 0.0, 0.5)
    with pytest.raises(_lib.GbError, match="theta must lie"):
        gn.solve_transient(2, 0.1, 1.5)
