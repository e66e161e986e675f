"""Exodus II results files (goma_gb300/exodus.py), read back with SciPy's
NetCDF reader: the DOF map equals the oracle's, the file holds the
reference's variable names (VX, VY, VZ, T, Y<k>; P1 pressure as P_E0..),
the mesh, node sets and every record, and the reference's own converged
cavity solution comes out with its lid velocity on the lid nodes."""
import os

import numpy as np
import pytest

import oracle
from goma_gb300 import exodus as ex
from goma_gb300 import problem as pb
from tests import golden_cases as gc


def _names(var):
    return [b"".join(r).decode().rstrip("\x00") for r in var[:]]


@pytest.mark.parametrize("prob_fn", [
    lambda: pb.lid_cavity_2d(3),
    lambda: pb.carreau_step_2d(4, 2, 10.0),
    lambda: pb.boussinesq_cube_3d(2, 1e4, 0.71),
    lambda: pb.reacting_channel_3d(2, 2, 1),
], ids=["cavity2d", "carreau2d", "bouss3d", "reacting3d"])
def test_round_trip(tmp_path, prob_fn):
    from scipy.io import netcdf_file
    prob = prob_fn()
    o = oracle.Oracle(prob)
    fu = ex.first_unknowns(prob)
    assert np.array_equal(fu, o.first_unknown(prob.mesh.num_nodes))
    rng = np.random.default_rng(1)
    xs = [rng.normal(size=o.N) for _ in range(3)]
    path = os.path.join(tmp_path, "sol.exo")
    ex.write_exodus(path, prob, xs, times=[0.5, 1.0, 2.0])
    f = netcdf_file(path, "r", mmap=False)
    try:
        dim = prob.dim
        assert f.dimensions["num_dim"] == dim
        assert f.dimensions["num_nodes"] == prob.mesh.num_nodes
        assert f.dimensions["num_elem"] == prob.mesh.num_elems
        assert f.variables["connect1"].elem_type == (b"QUAD9" if dim == 2 else b"HEX27")
        assert np.array_equal(f.variables["connect1"][:], prob.mesh.conn + 1)
        for a, c in zip("xyz", range(dim)):
            assert np.array_equal(f.variables["coord" + a][:], prob.mesh.coords[:, c])
        assert list(f.variables["time_whole"][:]) == [0.5, 1.0, 2.0]
        nodal_names = _names(f.variables["name_nod_var"])
        elem_names = _names(f.variables["name_elem_var"])
        want = ["VX", "VY", "VZ"][:dim] + (["T"] if prob.energy else []) + [
            "Y%d" % k for k in range(prob.num_species)]
        assert nodal_names == want
        assert elem_names == ["P_E%d" % k for k in range(dim + 1)]
        cent = prob.mesh.conn[:, 8 if dim == 2 else 20]
        for step, x in enumerate(xs):
            for k in range(len(nodal_names)):
                got = f.variables["vals_nod_var%d" % (k + 1)][step]
                assert np.array_equal(got, x[fu[:-1] + k])
            for k in range(dim + 1):
                got = f.variables["vals_elem_var%deb1" % (k + 1)][step]
                assert np.array_equal(got, x[fu[cent] + len(nodal_names) + k])
        for k, s in enumerate(prob.mesh.node_sets):
            assert np.array_equal(f.variables["node_ns%d" % (k + 1)][:], np.asarray(s) + 1)
    finally:
        f.close()


def test_reference_cavity_solution_fields(tmp_path):
    """The reference's converged 4x4 cavity: VX on every node of a U_BC card
    is that card's value, the later card winning where node sets share a
    corner (the deck order the reference applies them in)."""
    from scipy.io import netcdf_file
    g, case = gc.load("cav2d_4x4_solve")
    prob = gc.problem_from_case(case)
    path = os.path.join(tmp_path, "cavity.exo")
    ex.write_exodus(path, prob, g["x_converged"])
    nodal, elem = ex.split_solution(prob, g["x_converged"])
    f = netcdf_file(path, "r", mmap=False)
    try:
        vx = f.variables["vals_nod_var1"][0]
        assert np.array_equal(vx, nodal[0])
        want = {}
        for var, ns, value in prob.bcs:
            if var == 0:  # U_BC cards
                for n in prob.mesh.node_sets[ns - 1]:
                    want[int(n)] = value
        assert len(want) > 0 and max(want.values()) == 1.0
        nodes = np.array(sorted(want))
        assert np.allclose(vx[nodes], [want[n] for n in nodes], atol=1e-12)
    finally:
        f.close()


def test_wrong_length_is_rejected():
    prob = pb.lid_cavity_2d(2)
    with pytest.raises(ValueError, match="unknowns"):
        ex.split_solution(prob, np.zeros(5))
