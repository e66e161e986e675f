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
