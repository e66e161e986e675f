"""GPU Newton (assembly + row-sum scaling + ILU(0)-GMRES in FP64, FP32
inner GMRES inside FP64 refinement, and FP64 flexible GMRES with the
ILU(0) factorised and applied in FP32) against the reference's converged
solutions: fields within 1e-8 relative of the reference's FP64 Newton
solution."""
import numpy as np
import pytest

import oracle
from goma_gb300 import problem as pb
from goma_gb300.newton import GomaNewton
from tests import golden_cases as gc

pytestmark = pytest.mark.gpu
TOL_X = 1e-8
PRECISIONS = {"fp64": {}, "fp32_refined": {"fp32_inner": True},
              "fp32_preconditioner": {"fp32_preconditioner": True}}


@pytest.mark.parametrize("ordering", [0, 1], ids=["ilu_natural", "ilu_multicolour"])
@pytest.mark.parametrize("precision", list(PRECISIONS))
@pytest.mark.parametrize("name", gc.names("solve"))
def test_gpu_newton_matches_reference_solution(name, precision, ordering):
    """Both ILU(0) node orders: the preconditioner changes the Krylov
    iterates, never the converged Newton solution."""
    g, case = gc.load(name)
    gn = GomaNewton(gc.problem_from_case(case))
    gn.set_ilu_ordering(ordering)
    x0 = g["x0"] if "x0" in g else None
    x, conv, st = gn.solve_nonlinear_problem(x0, residual_tol=1e-11, linear_tol=1e-10,
                                             max_newton=30, **PRECISIONS[precision])
    assert conv, st
    xc = g["x_converged"]
    assert np.abs(x - xc).max() <= TOL_X * np.abs(xc).max()


@pytest.mark.parametrize("precision", list(PRECISIONS))
@pytest.mark.parametrize("name", gc.names("solve", compact=True))
def test_gpu_newton_matches_reference_solution_at_benchmark_size(name, precision):
    """The 32 x 32 lid-driven cavity at Re 100 (the benchmark size, 11,522
    unknowns) from rest to the scaled residual 1e-10, against the reference's
    converged fields, with the reference's solver settings (ILU(0) in its
    node order, GMRES(30))."""
    g, case = gc.load(name)
    gn = GomaNewton(gc.problem_from_case(case))
    gn.set_ilu_ordering(0)
    x, conv, st = gn.solve_nonlinear_problem(None, residual_tol=case["tol"], linear_tol=1e-10,
                                             max_newton=30, krylov_dim=30, max_linear_its=3000,
                                             **PRECISIONS[precision])
    assert conv, st
    xc = g["x_converged"]
    assert np.abs(x - xc).max() <= TOL_X * np.abs(xc).max()


def test_gpu_linear_solve_drop_in():
    """gb_linear_solve on the reference-scaled MSR system matches a direct
    solve of the same system (oracle band LU via one Newton correction)."""
    prob = pb.lid_cavity_2d(6, 100.0)
    o = oracle.Oracle(prob)
    gn = GomaNewton(prob)
    x = o.dirichlet_init(np.random.default_rng(0).uniform(-0.5, 0.5, o.N))
    R, a, _ = o.matrix_fill(x)
    a_s, R_s, _ = o.row_sum_scale(a, R)
    dx, its, rr = gn.linear_solve(a_s, R_s, linear_tol=1e-12, max_linear_its=2000)
    assert rr <= 1e-12
    # residual of the scaled system
    ija = o.ija()
    N = o.N
    Ax = a_s[:N] * dx
    for i in range(N):
        Ax[i] += np.dot(a_s[ija[i]:ija[i + 1]], dx[ija[ija[i]:ija[i + 1]]])
    assert np.abs(Ax - R_s).max() <= 1e-9 * np.abs(R_s).max()


def test_gpu_newton_larger_cavity_against_oracle():
    prob = pb.lid_cavity_2d(16, 100.0)
    o = oracle.Oracle(prob)
    xo, it, _ = o.newton(o.dirichlet_init(np.zeros(o.N)), 30, 1e-11)
    assert it > 0
    gn = GomaNewton(prob)
    for fp32 in (False, True):
        x, conv, st = gn.solve_nonlinear_problem(residual_tol=1e-11, linear_tol=1e-10,
                                                 fp32_inner=fp32)
        assert conv
        assert np.abs(x - xo).max() <= TOL_X * np.abs(xo).max()


@pytest.mark.parametrize("case", ["cavity2d_12", "bouss3d_4"])
def test_gpu_triangular_solve_modes_agree(case):
    """Sync-free ILU(0) sweeps and the level-scheduled graph apply the same
    preconditioner (summation order differs), so a fixed number of GMRES
    iterations gives the same correction to rounding."""
    prob = (pb.lid_cavity_2d(12, 100.0) if case.startswith("cavity")
            else pb.boussinesq_cube_3d(4, 1e4, 0.71))
    gn = GomaNewton(prob)
    o = oracle.Oracle(prob)
    x = o.dirichlet_init(np.random.default_rng(1).uniform(-0.5, 0.5, o.N))
    R, a = gn.matrix_fill_full(x)
    a_s, R_s, _ = o.row_sum_scale(a, R)
    out = []
    for mode in (1, 0, 0):
        gn.set_triangular_solve(mode)
        dx, its, rr = gn.linear_solve(a_s, R_s, linear_tol=1e-30, max_linear_its=8)
        assert its == 8
        out.append(dx)
    scale = np.abs(out[0]).max()
    assert np.abs(out[1] - out[0]).max() <= 1e-10 * scale
    assert np.array_equal(out[2], out[1])   # the sync-free sweeps are deterministic


@pytest.mark.parametrize("name", ["cav2d_3x2_pert", "bfs2d_4x2_carreau", "box3d_2x2x2_bouss",
                                  "box3d_2x2x2_species"])
def test_gpu_ilu0_factors_match_oracle(name):
    """The GPU's node-block ILU(0) (FP64 and FP32) equals the oracle's
    row-by-row ILU(0) of the same row-scaled reference Jacobian, pivot
    floor included (the Carreau channel without a pressure datum hits it).
    FP32 tolerance: single-precision rounding (6e-8) amplified by the
    floored pivots (1e-4) of that channel."""
    g, case = gc.load(name)
    prob = gc.problem_from_case(case)
    o = oracle.Oracle(prob)
    gn = GomaNewton(prob)
    a_s, _, _ = o.row_sum_scale(g["a"], g["R"])
    ref = o.ilu0(a_s, tau=1e-4)
    ija = o.ija()
    for fp32, tol in ((False, 1e-10), (True, 2e-3)):
        lu = gn.ilu0_factors(a_s, fp32=fp32)
        assert gc.msr_row_scaled_error(ija, lu, ref) < tol, fp32


@pytest.mark.parametrize("trsv", [0, 1], ids=["sync_free", "level_graph"])
def test_multicolour_ilu_solves_the_cube(trsv):
    """The multicoloured ILU(0) preconditioner on a 6^3 Boussinesq cube (both
    triangular-solve modes): GMRES reaches the same Newton solution as the
    reference-order ILU(0)."""
    prob = pb.boussinesq_cube_3d(6, 1e4, 0.71)
    sols = []
    for ordering in (0, 1):
        gn = GomaNewton(prob)
        gn.set_triangular_solve(trsv)
        gn.set_ilu_ordering(ordering)
        x, conv, st = gn.solve_nonlinear_problem(residual_tol=1e-10, linear_tol=1e-9,
                                                 max_newton=30, max_linear_its=4000)
        assert conv, (ordering, st)
        sols.append(x)
        gn.close()
    assert np.abs(sols[0] - sols[1]).max() <= TOL_X * np.abs(sols[0]).max()


def test_gpu_krylov_counts_match_oracle_gmres():
    """With the reference's solver settings (ILU(0) in its node order,
    GMRES(30), every linear solve to 1e-8) the GPU Newton loop takes the
    same Newton steps as the oracle's Newton with its restated
    ILU(0)-GMRES(30), the same Krylov iterations up to the rounding of the
    two Gram-Schmidt variants (classical with one reorthogonalisation on the
    GPU, modified in the oracle), and reaches the same fields."""
    prob = pb.boussinesq_cube_3d(3, 1e4, 0.71)
    o = oracle.Oracle(prob)
    x0 = o.dirichlet_init(np.zeros(o.N))
    xo, ito, lino, _ = o.newton_gmres(x0, 40, 1e-10, linear_tol=1e-8, krylov=30,
                                      max_linear_its=4000)
    assert ito > 0
    gn = GomaNewton(prob)
    x, conv, st = gn.solve_nonlinear_problem(x0, residual_tol=1e-10, linear_tol=1e-8,
                                             krylov_dim=30, forcing=0, max_newton=40,
                                             max_linear_its=4000)
    assert conv
    assert abs(st["newton_its"] - ito) <= 1
    assert abs(st["linear_its"] - lino) <= max(3, 0.1 * lino)
    assert np.abs(x - xo).max() <= TOL_X * np.abs(xo).max()


@pytest.mark.parametrize("fp32", [False, True], ids=["fp64", "fp32_refined"])
def test_gpu_factorization_reuse(fp32):
    """The reference's "Matrix Factorization Reuse" choices: CALC factors at
    every Newton step, REUSE keeps the last factors across calls (here a
    continuation-like call at a nearby Rayleigh number factors nothing),
    PER_SOLVE factors once per call.  Every mode converges to the fields of
    the CALC solve."""
    def solve(ra, x0, reuse, gn=None):
        if gn is None:
            gn = GomaNewton(pb.boussinesq_cube_3d(3, ra, 0.71))
        x, conv, st = gn.solve_nonlinear_problem(
            x0, residual_tol=1e-10, linear_tol=1e-9, krylov_dim=60, max_newton=30,
            max_linear_its=4000, fp32_inner=fp32, factorization_reuse=reuse)
        assert conv, (ra, reuse, st)
        return gn, x, st

    gn, xc, st = solve(1e4, None, 0)
    assert st["factorizations"] == st["newton_its"] > 0
    # the next parameter value with the last factors of the converged solve
    m = gn.problem.material
    m.momentum_source = (0.0, 0.0, -1.2e4 * 0.71)
    gn.set_material(m)
    _, xr, st = solve(1.2e4, xc, 2, gn)
    assert st["factorizations"] == 0 and st["newton_its"] > 0
    _, xref, _ = solve(1.2e4, xc, 0)
    assert np.abs(xr - xref).max() <= TOL_X * np.abs(xref).max()
    _, xp, st = solve(1e4, None, 1)
    assert st["factorizations"] == 1
    assert np.abs(xp - xc).max() <= TOL_X * np.abs(xc).max()


def test_gpu_long_gmres_restart_matches_short_one():
    """A restart length beyond 63 (its Gram-Schmidt coefficients need more
    than two warps in the final reduction) solves the same Newton system to
    the same solution as GMRES(30)."""
    prob = pb.boussinesq_cube_3d(4, 1e4, 0.71)
    o = oracle.Oracle(prob)
    x = o.dirichlet_init(np.random.default_rng(3).uniform(-0.5, 0.5, o.N))
    R, a, _ = o.matrix_fill(x)
    a_s, R_s, _ = o.row_sum_scale(a, R)
    gn = GomaNewton(prob)
    dx30, its30, rr30 = gn.linear_solve(a_s, R_s, linear_tol=1e-11, max_linear_its=4000,
                                        krylov_dim=30)
    dx150, its150, rr150 = gn.linear_solve(a_s, R_s, linear_tol=1e-11, max_linear_its=4000,
                                           krylov_dim=150)
    assert rr30 <= 1e-11 and rr150 <= 1e-11
    assert its150 <= its30
    assert np.abs(dx150 - dx30).max() <= 1e-8 * np.abs(dx30).max()
