"""The CPU oracle against golden vectors produced by the reference itself
(tests/golden/make_golden.py runs the unmodified reference C): sparsity
bit-exact, R and J within 1e-12 (row-scaled), converged Newton fields
within 1e-8 relative."""
import numpy as np
import pytest

import oracle
from tests import golden_cases as gc

TOL_RJ = 1e-12
TOL_X = 1e-8


@pytest.mark.parametrize("name", gc.names("assemble"))
def test_oracle_assembly_matches_reference(name):
    g, case = gc.load(name)
    o = oracle.Oracle(gc.problem_from_case(case))
    ija = o.ija()
    assert np.array_equal(ija, g["ija"]), "MSR pattern differs from the reference"
    R, a, st = o.matrix_fill(g["x"])
    assert st == 0
    assert gc.msr_row_scaled_error(ija, a, g["a"]) < TOL_RJ
    assert np.abs(R - g["R"]).max() <= TOL_RJ * np.abs(g["R"]).max()


@pytest.mark.parametrize("name", gc.names("solve"))
def test_oracle_newton_matches_reference(name):
    g, case = gc.load(name)
    o = oracle.Oracle(gc.problem_from_case(case))
    assert np.array_equal(o.ija(), g["ija"])
    x0 = g["x0"] if "x0" in g else o.dirichlet_init(np.zeros(o.N))
    x, it, _ = o.newton(x0, 40, 1e-12)
    assert it > 0
    xc = g["x_converged"]
    assert np.abs(x - xc).max() <= TOL_X * np.abs(xc).max()


@pytest.mark.parametrize("name", gc.names("assemble", compact=True))
def test_oracle_assembly_matches_reference_at_benchmark_size(name):
    """The 32 x 32 lid-driven cavity (the benchmark size): the whole pattern
    (hash), every residual entry and a seeded sample of Jacobian rows."""
    g, case = gc.load(name)
    o = oracle.Oracle(gc.problem_from_case(case))
    R, a, st = o.matrix_fill(g["x"])
    assert st == 0
    jerr, rerr = gc.compact_rows_check(g, o.ija(), a, R)
    assert jerr < TOL_RJ and rerr <= TOL_RJ


@pytest.mark.parametrize("name", gc.names("solve", compact=True))
def test_oracle_newton_matches_reference_at_benchmark_size(name):
    import hashlib
    g, case = gc.load(name)
    o = oracle.Oracle(gc.problem_from_case(case))
    ija = o.ija()
    assert hashlib.sha256(ija.astype("<i4").tobytes()).hexdigest() == str(g["ija_sha256"])
    x, it, _ = o.newton(o.dirichlet_init(np.zeros(o.N)), 40, case["tol"])
    assert it > 0
    xc = g["x_converged"]
    assert np.abs(x - xc).max() <= TOL_X * np.abs(xc).max()


@pytest.mark.parametrize("name", gc.names("assemble", transient=True))
def test_oracle_transient_assembly_matches_reference(name):
    """The first assembly of a time step with a seeded state and time
    derivative: mass terms of xdot in R, their (1 + 2 theta) / dt sensitivity
    in J (momentum, energy, species)."""
    g, case = gc.load(name)
    o = oracle.Oracle(gc.problem_from_case(case))
    assert np.array_equal(o.ija(), g["ija"])
    dt, theta = g["delta_t_theta"]
    R, a, st = o.matrix_fill(g["x"], xdot=g["xdot"], delta_t=dt, theta=theta)
    assert st == 0
    assert gc.msr_row_scaled_error(g["ija"], a, g["a"]) < TOL_RJ
    assert np.abs(R - g["R"]).max() <= TOL_RJ * np.abs(g["R"]).max()


@pytest.mark.parametrize("name", gc.names("transient"))
def test_oracle_transient_run_matches_reference(name):
    """The reference's fixed-step time loop from rest: three backward-Euler
    steps, then Crank-Nicolson with its second-order predictor; the solution
    after every step."""
    g, case = gc.load(name)
    tr = case["transient"]
    o = oracle.Oracle(gc.problem_from_case(case))
    xs = o.transient_run(np.zeros(o.N), tr["steps"], tr["dt"], tr["theta"], tol=case["tol"])
    ref = g["x_steps"]
    assert len(xs) == len(ref)
    for k, (x, xr) in enumerate(zip(xs, ref)):
        assert np.abs(x - xr).max() <= TOL_X * np.abs(xr).max(), k


def test_oracle_mesh_generator_matches_package():
    from goma_gb300.problem import mesh_from_spec
    for spec in ["quad9 3 2 1.5 1 0.15 7", "hex27 2 1 3 1 0.5 1.5 0.12 9", "quad9 5 4 2 1"]:
        c, k, s = oracle.mesh_from_spec(spec)
        m = mesh_from_spec(spec)
        assert np.array_equal(c, m.coords)
        assert np.array_equal(k, m.conn)
        assert all(np.array_equal(a, b) for a, b in zip(s, m.node_sets))


def test_oracle_detects_inverted_element():
    from goma_gb300 import problem as pb
    prob = pb.lid_cavity_2d(2)
    # mirror element 0 by swapping two corner nodes: negative Jacobian
    conn = prob.mesh.conn.copy()
    conn[0, [0, 1]] = conn[0, [1, 0]]
    prob.mesh.conn = conn
    o = oracle.Oracle(prob)
    _, _, st = o.matrix_fill(np.zeros(o.N))
    assert st == -1


def test_oracle_ilu0_reproduces_matrix_on_pattern():
    """ILU(0) property: (L U)_ij = A_ij on the sparsity pattern (no pivot
    floor hit), on the reference's own row-scaled Jacobian."""
    sp = pytest.importorskip("scipy.sparse")
    g, case = gc.load("cav2d_3x2_pert")
    o = oracle.Oracle(gc.problem_from_case(case))
    a_s, _, _ = o.row_sum_scale(g["a"], g["R"])
    lu = o.ilu0(a_s, tau=0.0)
    ija = o.ija()
    N = o.N

    def to_csr(v):
        rows, cols, vals = list(range(N)), list(range(N)), list(v[:N])
        for i in range(N):
            for k in range(ija[i], ija[i + 1]):
                rows.append(i)
                cols.append(ija[k])
                vals.append(v[k])
        return sp.csr_matrix((vals, (rows, cols)), shape=(N, N))

    A = to_csr(a_s)
    F = to_csr(lu)
    Lm = sp.tril(F, -1) + sp.identity(N)
    Um = sp.triu(F)
    P = (Lm @ Um).tocsr()
    Ad = A.toarray()
    Pd = P.toarray()
    mask = A.toarray() != 0
    mask |= to_csr(np.ones_like(a_s)).toarray() != 0
    assert np.abs((Pd - Ad)[mask]).max() <= 1e-12 * np.abs(Ad).max()
