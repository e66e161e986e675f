"""The multicoloured node order of the GPU-friendly ILU(0) variant, checked
on the host: a permutation of the nodes whose renumbered CSR pattern is the
original one entry for entry (the value map hits every original entry
once), with few dependency levels, and every centroid (pressure) node after
all other nodes."""
import ctypes

import numpy as np
import pytest

from goma_gb300 import _lib
from goma_gb300 import problem as pb
from goma_gb300.newton import msr_pattern_host


def _csr_from_msr(ija, N):
    rowptr = np.zeros(N + 1, np.int64)
    colidx = []
    for i in range(N):
        c = sorted([i] + list(ija[ija[i]:ija[i + 1]]))
        colidx.extend(c)
        rowptr[i + 1] = rowptr[i] + len(c)
    return rowptr, np.array(colidx, np.int64)


@pytest.mark.parametrize("prob_fn", [
    lambda: pb.lid_cavity_2d(4),
    lambda: pb.carreau_step_2d(5, 2, 10.0),
    lambda: pb.boussinesq_cube_3d(3),
    lambda: pb.reacting_channel_3d(2, 2, 1),
    lambda: pb.batch_sweep_2d(3, seed=2, nmin=2, nmax=3).problem,
], ids=["cavity2d", "carreau2d", "bouss3d", "reacting3d", "batch2d"])
def test_multicolour_order_and_permuted_pattern(prob_fn):
    prob = prob_fn()
    L = _lib.load()
    desc, keep = pb.make_desc(prob)
    ija = msr_pattern_host(prob)
    N = int(ija[0]) - 1
    nnz = len(ija) - 1
    nn = prob.mesh.num_nodes
    perm = np.empty(nn, np.int32)
    ncol = ctypes.c_int()
    umap = np.empty(N, np.int32)
    rp = np.empty(N + 1, np.int64)
    ci = np.empty(nnz, np.int32)
    vm = np.empty(nnz, np.int64)
    P = lambda a, t: a.ctypes.data_as(ctypes.POINTER(t))  # noqa: E731
    _lib.check(L.gb_ilu_permutation_host(ctypes.byref(desc), P(perm, ctypes.c_int),
                                         ctypes.byref(ncol), P(umap, ctypes.c_int),
                                         P(rp, ctypes.c_longlong), P(ci, ctypes.c_int),
                                         P(vm, ctypes.c_longlong)))
    del keep
    assert np.array_equal(np.sort(perm), np.arange(nn))
    assert np.array_equal(np.sort(umap), np.arange(N))
    orp, oci = _csr_from_msr(ija, N)
    assert rp[-1] == nnz
    # every permuted entry is the original entry (umap[i'], umap[j'])
    rows_new = np.repeat(np.arange(N), np.diff(rp))
    old_i = umap[rows_new]
    old_j = umap[ci]
    assert np.all(vm >= orp[old_i]) and np.all(vm < orp[old_i + 1])
    assert np.array_equal(oci[vm], old_j)
    assert np.array_equal(np.sort(vm), np.arange(nnz))
    for i in range(N):  # ascending columns in every permuted row
        assert np.all(np.diff(ci[rp[i]:rp[i + 1]]) > 0)
    # node dependency levels of the permuted pattern (the unknowns of a node
    # stay contiguous and in node order)
    old_node = _old_node_of_unknowns(N, prob)
    new_node = perm[old_node[umap]]
    assert np.all(np.diff(new_node) >= 0)
    level = np.zeros(nn, np.int64)
    for i in range(N):
        n = new_node[i]
        lower = new_node[ci[rp[i]:rp[i + 1]]]
        lower = lower[lower < n]
        if lower.size:
            level[n] = max(level[n], level[lower].max() + 1)
    assert level.max() + 1 <= ncol.value
    assert ncol.value <= (12 if prob.dim == 2 else 32)
    # centroid (pressure) nodes come after every other node
    counts = np.bincount(old_node, minlength=nn)
    cent_new = perm[counts > counts.min()]
    other_new = perm[counts == counts.min()]
    assert cent_new.min() > other_new.max()


def _old_node_of_unknowns(N, prob):
    """Node of every original unknown: the nodal fields at every node, the
    P1 pressures after them at element centroids (node-major order)."""
    nn = prob.mesh.num_nodes
    dim = prob.dim
    nvn = dim + (1 if prob.energy else 0) + prob.num_species
    cent = set(prob.mesh.conn[:, 8 if dim == 2 else 20].tolist())
    counts = np.array([nvn + (dim + 1 if n in cent else 0) for n in range(nn)])
    assert counts.sum() == N
    return np.repeat(np.arange(nn), counts)


@pytest.mark.parametrize("ordering", [0, 1], ids=["natural", "multicolour"])
@pytest.mark.parametrize("prob_fn", [
    lambda: pb.lid_cavity_2d(4),
    lambda: pb.boussinesq_cube_3d(3),
    lambda: pb.reacting_channel_3d(2, 2, 1),
], ids=["cavity2d", "bouss3d", "reacting3d"])
def test_sweep_order_is_a_level_sorted_permutation_of_each_segment(prob_fn, ordering):
    """The order in which the sync-free sweeps read a row's off-node entries
    (checked here on the host before any sweep uses it): within every
    row's lower segment [row start, own block) and upper segment (after the
    own block, row end) it is a permutation of the segment's positions, it
    stays inside the segment, and it takes the neighbour nodes by ascending
    dependency level (forward levels for the lower, backward for the
    upper segment)."""
    prob = prob_fn()
    L = _lib.load()
    desc, keep = pb.make_desc(prob)
    ija = msr_pattern_host(prob)
    N = int(ija[0]) - 1
    nnz = len(ija) - 1
    nn = prob.mesh.num_nodes
    P = lambda a, t: a.ctypes.data_as(ctypes.POINTER(t))  # noqa: E731
    rel = np.empty(nnz, np.uint16)
    lev = np.empty(nn, np.int32)
    levu = np.empty(nn, np.int32)
    _lib.check(L.gb_sweep_order_host(ctypes.byref(desc), ordering, P(rel, ctypes.c_ushort),
                                     P(lev, ctypes.c_int), P(levu, ctypes.c_int)))
    if ordering == 0:
        rp, ci = _csr_from_msr(ija, N)
        node = _old_node_of_unknowns(N, prob)
    else:
        perm = np.empty(nn, np.int32)
        umap = np.empty(N, np.int32)
        rp = np.empty(N + 1, np.int64)
        ci32 = np.empty(nnz, np.int32)
        _lib.check(L.gb_ilu_permutation_host(ctypes.byref(desc), P(perm, ctypes.c_int), None,
                                             P(umap, ctypes.c_int), P(rp, ctypes.c_longlong),
                                             P(ci32, ctypes.c_int), None))
        ci = ci32.astype(np.int64)
        node = perm[_old_node_of_unknowns(N, prob)[umap]]
    del keep
    for i in range(N):
        n = node[i]
        cols = ci[rp[i]:rp[i + 1]]
        own = np.flatnonzero(node[cols] == n)
        lo0, lo1 = rp[i], rp[i] + own[0]
        up0, up1 = rp[i] + own[-1] + 1, rp[i + 1]
        for s0, s1, lv, below in ((lo0, lo1, lev, True), (up0, up1, levu, False)):
            r = rel[s0:s1].astype(np.int64)
            assert np.array_equal(np.sort(r), np.arange(s1 - s0)), i
            nodes = node[ci[s0 + r]]
            assert np.all(nodes < n) if below else np.all(nodes > n)
            assert np.all(np.diff(lv[nodes]) >= 0), i
