"""A batch of independent 2-D cavity / channel problems with different
Reynolds numbers, held in one context as a disjoint union with per-element
densities: its assembly and its Newton solution equal, member by member,
the oracle's for each problem on its own."""
import numpy as np
import pytest

import oracle
from goma_gb300 import problem as pb
from goma_gb300.newton import GomaNewton

pytestmark = pytest.mark.gpu


def _msr_dense(ija, a, lo, hi):
    """Rows/columns [lo, hi) of an MSR matrix as a dense block."""
    D = np.zeros((hi - lo, hi - lo))
    for i in range(lo, hi):
        D[i - lo, i - lo] = a[i]
        for k in range(ija[i], ija[i + 1]):
            j = ija[k]
            assert lo <= j < hi, "coupling between members"
            D[i - lo, j - lo] = a[k]
    return D


@pytest.fixture(scope="module")
def batch():
    b = pb.batch_sweep_2d(6, seed=3, nmin=2, nmax=5, re_min=10.0, re_max=100.0)
    gn = GomaNewton(b.problem)
    gn.set_element_density(b.elem_re)
    fu = np.empty(b.problem.mesh.num_nodes + 1, np.int32)
    import ctypes
    from goma_gb300 import _lib
    _lib.check(gn._L.gb_first_unknown(gn.h, fu.ctypes.data_as(ctypes.POINTER(ctypes.c_int))))
    return b, gn, fu


def test_batch_assembly_equals_members(batch):
    b, gn, fu = batch
    rng = np.random.default_rng(8)
    x = gn.dirichlet_init(rng.uniform(-1, 1, gn.N))
    R, a = gn.matrix_fill_full(x)
    ija = gn.msr_pattern()
    for p, mb in enumerate(b.members):
        lo, hi = fu[mb.nodes[0]], fu[mb.nodes[1]]
        o = oracle.Oracle(pb.batch_member_problem(b, p))
        assert o.N == hi - lo
        Ro, ao, st = o.matrix_fill(x[lo:hi])
        assert st == 0
        Do = _msr_dense(o.ija(), ao, 0, o.N)
        Dg = _msr_dense(ija, a, lo, hi)
        scale = np.maximum(np.abs(Do).max(axis=1), 1e-300)
        assert (np.abs(Dg - Do).max(axis=1) / scale).max() < 1e-12, p
        assert np.abs(R[lo:hi] - Ro).max() <= 1e-12 * np.abs(Ro).max(), p


def test_batch_newton_equals_members(batch):
    b, gn, fu = batch
    x, conv, st = gn.solve_nonlinear_problem(residual_tol=1e-10, linear_tol=1e-10,
                                             max_newton=30, max_linear_its=3000)
    assert conv
    for p, mb in enumerate(b.members):
        lo, hi = fu[mb.nodes[0]], fu[mb.nodes[1]]
        o = oracle.Oracle(pb.batch_member_problem(b, p))
        xo, its, _ = o.newton(o.dirichlet_init(np.zeros(o.N)))
        assert its >= 0
        assert np.abs(x[lo:hi] - xo).max() <= 1e-8 * np.abs(xo).max(), p


def test_batch_newton_fp32_preconditioner_equals_members(batch):
    """The batched GMRES in the FP32-preconditioner mode (one flexible GMRES
    per member, the block-diagonal ILU(0) in FP32): every member's solution
    equals the oracle's for that problem on its own."""
    b, gn, fu = batch
    x, conv, st = gn.solve_nonlinear_problem(residual_tol=1e-10, linear_tol=1e-10,
                                             max_newton=30, max_linear_its=3000,
                                             fp32_preconditioner=True)
    assert conv
    for p, mb in enumerate(b.members):
        lo, hi = fu[mb.nodes[0]], fu[mb.nodes[1]]
        o = oracle.Oracle(pb.batch_member_problem(b, p))
        xo, its, _ = o.newton(o.dirichlet_init(np.zeros(o.N)))
        assert its >= 0
        assert np.abs(x[lo:hi] - xo).max() <= 1e-8 * np.abs(xo).max(), p
