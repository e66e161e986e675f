"""The threaded CPU assembly that the benchmark's reference arm times
(oracle.ParallelFill: colour-disjoint element chunks into one shared MSR
array) gives the serial oracle's R and Jacobian, and its colouring leaves no
two elements of a colour sharing a node."""
import numpy as np
import pytest

import oracle
from goma_gb300 import problem as pb


@pytest.mark.parametrize("make", [lambda: pb.boussinesq_cube_3d(3, 1e5, 0.71),
                                  lambda: pb.lid_cavity_2d(5, 100.0)])
def test_parallel_fill_matches_serial_fill(make):
    prob = make()
    o = oracle.Oracle(prob)
    x = o.dirichlet_init(np.random.default_rng(4).uniform(-1, 1, o.N))
    R, a, st = o.matrix_fill(x)
    assert st == 0
    pf = oracle.ParallelFill(o, 3)
    try:
        assert pf(x) == 0
        assert pf(x) == 0   # a second call starts from zero again
        assert np.abs(pf.R - R).max() <= 1e-13 * np.abs(R).max()
        assert np.abs(pf.a - a).max() <= 1e-13 * np.abs(a).max()
        conn = np.asarray(prob.mesh.conn)
        seen = set()
        for col in pf.chunks:
            els = np.concatenate(col)
            nodes = conn[els].ravel()
            assert len(np.unique(nodes)) == nodes.size
            seen.update(els.tolist())
        assert seen == set(range(prob.mesh.num_elems))
    finally:
        pf.close()
