"""GPU assembly (libgbnewton.so through its C ABI) against the reference's
golden vectors and the CPU oracle.  Residual and Jacobian entries must
agree within 1e-12 relative (per row, scaled by the row's largest
reference entry); the MSR pattern bit for bit."""
import numpy as np
import pytest

import oracle
from goma_gb300 import problem as pb
from goma_gb300.newton import GomaNewton
from tests import golden_cases as gc

pytestmark = pytest.mark.gpu
TOL = 1e-12


@pytest.mark.parametrize("name", gc.names("assemble"))
def test_gpu_assembly_matches_reference(name):
    g, case = gc.load(name)
    gn = GomaNewton(gc.problem_from_case(case))
    assert np.array_equal(gn.msr_pattern(), g["ija"])
    R, a = gn.matrix_fill_full(g["x"])
    assert gc.msr_row_scaled_error(g["ija"], a, g["a"]) < TOL
    assert np.abs(R - g["R"]).max() <= TOL * np.abs(g["R"]).max()


def _random_state(o, seed, scale=1.0):
    rng = np.random.default_rng(seed)
    return rng.uniform(-scale, scale, o.N)


@pytest.mark.parametrize("prob_fn", [
    lambda: pb.lid_cavity_2d(8, 100.0, mesh=pb.box_mesh(2, 8, 6, 1, 1.3, 1.0, amp=0.15, seed=3)),
    lambda: pb.carreau_step_2d(9, 4, 30.0, mesh=pb.box_mesh(2, 9, 4, 1, 3.0, 1.0, amp=0.1,
                                                            seed=5)),
    lambda: pb.boussinesq_cube_3d(3, 1e4, 0.71, mesh=pb.box_mesh(3, 3, 3, 3, amp=0.12, seed=2)),
    lambda: pb.Problem(pb.box_mesh(3, 2, 3, 2, 1.0, 1.5, 0.7, amp=0.1, seed=8),
                       pb.Material(density=2.0, viscosity_model=pb.VISC_CARREAU, mu0=1.5,
                                   mu_inf=0.05, lam=0.7, aexp=2.0, nexp=0.4,
                                   heat_capacity=1.3, conductivity=0.8,
                                   momentum_source_model=pb.SOURCE_BOUSSINESQ,
                                   momentum_source=(0.0, -9.0, -3.0), volume_expansion=0.5,
                                   reference_temperature=0.2),
                       True, list(pb.HEATED3D_BCS), (3, 0.0)),
], ids=["cavity2d_8x6_pert", "carreau2d_9x4_pert", "bouss3d_3x3x3_pert", "carreau_t3d_2x3x2"])
def test_gpu_assembly_matches_oracle(prob_fn):
    prob = prob_fn()
    o = oracle.Oracle(prob)
    gn = GomaNewton(prob)
    ija = o.ija()
    assert np.array_equal(gn.msr_pattern(), ija)
    x = _random_state(o, 17)
    Ro, ao, st = o.matrix_fill(x)
    assert st == 0
    R, a = gn.matrix_fill_full(x)
    assert gc.msr_row_scaled_error(ija, a, ao) < TOL
    assert np.abs(R - Ro).max() <= TOL * np.abs(Ro).max()


@pytest.mark.parametrize("path", [1, 4])
def test_gpu_reacting_channel_matches_oracle(path):
    """Channel flow with energy and two Arrhenius species on a perturbed
    mesh (the element kernels of the 64 x 64 x 32 reacting-channel workload,
    here at 3 x 2 x 2): flow rows from the automatic (sum-factorised) or the
    scalar kernel, species rows from the species kernel; unknowns drawn from
    [0.5, 1.5] so the temperature stays positive in exp(-E/T)."""
    prob = pb.reacting_channel_3d(3, 2, 2, seed=4,
                                  mesh=pb.box_mesh(3, 3, 2, 2, 2.0, 2.0, 1.0, amp=0.1, seed=6))
    o = oracle.Oracle(prob)
    gn = GomaNewton(prob)
    gn.set_assembly_path(path)
    ija = o.ija()
    assert np.array_equal(gn.msr_pattern(), ija)
    x = o.dirichlet_init(np.random.default_rng(29).uniform(0.5, 1.5, o.N))
    Ro, ao, st = o.matrix_fill(x)
    assert st == 0
    R, a = gn.matrix_fill_full(x)
    assert gc.msr_row_scaled_error(ija, a, ao) < TOL
    assert np.abs(R - Ro).max() <= TOL * np.abs(Ro).max()


def test_gpu_assembly_deterministic_and_residual_only():
    prob = pb.boussinesq_cube_3d(3, 1e5, 0.71)
    gn = GomaNewton(prob)
    x = np.random.default_rng(1).uniform(-1, 1, gn.N)
    R1, a1 = gn.matrix_fill_full(x)
    R2, a2 = gn.matrix_fill_full(x)
    R3, _ = gn.matrix_fill_full(x, jacobian=False)
    assert np.array_equal(R1, R2) and np.array_equal(a1, a2)
    assert np.array_equal(R1, R3)


def test_gpu_device_entry_point_matches_host_entry_point():
    import torch
    prob = pb.lid_cavity_2d(6, 50.0)
    gn = GomaNewton(prob)
    x = np.random.default_rng(4).uniform(-1, 1, gn.N)
    R_host, a_host = gn.matrix_fill_full(x)
    dx = torch.tensor(x, dtype=torch.float64, device="cuda")
    dR = torch.empty(gn.N, dtype=torch.float64, device="cuda")
    dv = torch.empty(gn.nnz, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    gn.matrix_fill_full_device(dx.data_ptr(), dR.data_ptr(), dv.data_ptr(), stream)
    torch.cuda.synchronize()
    gn.status()
    assert np.array_equal(dR.cpu().numpy(), R_host)
    assert np.array_equal(gn.csr_to_msr(dv.data_ptr()), a_host)


def test_gpu_msr_into_pinned_host_memory():
    """A pinned host buffer is filled directly by the conversion kernel; the
    result equals the staged copy into pageable memory bit for bit."""
    import ctypes

    import torch
    from goma_gb300 import _lib
    prob = pb.boussinesq_cube_3d(3, 1e4, 0.71, mesh=pb.box_mesh(3, 3, 3, 3, amp=0.1, seed=5))
    gn = GomaNewton(prob)
    x = gn.dirichlet_init(np.random.default_rng(6).uniform(-1, 1, gn.N))
    R_pg, a_pg = gn.matrix_fill_full(x)
    xh = torch.from_numpy(x.copy()).pin_memory()
    Rh = torch.empty(gn.N, dtype=torch.float64).pin_memory()
    ah = torch.empty(gn.msr_len, dtype=torch.float64).pin_memory()
    P = lambda t: ctypes.cast(t.data_ptr(), ctypes.POINTER(ctypes.c_double))  # noqa: E731
    _lib.check(gn._L.gb_matrix_fill_full(gn.h, P(xh), P(Rh), P(ah)))
    assert np.array_equal(Rh.numpy(), R_pg)
    assert np.array_equal(ah.numpy(), a_pg)


def test_gpu_reports_inverted_element():
    from goma_gb300 import _lib
    prob = pb.lid_cavity_2d(3)
    conn = prob.mesh.conn.copy()
    conn[4, [0, 2]] = conn[4, [2, 0]]
    prob.mesh.conn = conn
    gn = GomaNewton(prob)
    with pytest.raises(_lib.GbError, match="non-positive Jacobian"):
        gn.matrix_fill_full(np.zeros(gn.N))
    # the context stays usable
    gn2 = GomaNewton(pb.lid_cavity_2d(3))
    gn2.matrix_fill_full(np.zeros(gn2.N))


@pytest.mark.parametrize("prob_fn", [
    lambda: pb.boussinesq_cube_3d(3, 1e5, 0.71, mesh=pb.box_mesh(3, 3, 3, 3, amp=0.12, seed=2)),
    lambda: pb.Problem(pb.box_mesh(3, 2, 3, 2, 1.0, 1.5, 0.7, amp=0.1, seed=8),
                       pb.Material(density=2.0, viscosity_model=pb.VISC_CARREAU, mu0=1.5,
                                   mu_inf=0.05, lam=0.7, aexp=2.0, nexp=0.4,
                                   heat_capacity=1.3, conductivity=0.8,
                                   momentum_source_model=pb.SOURCE_BOUSSINESQ,
                                   momentum_source=(0.0, -9.0, -3.0), volume_expansion=0.5,
                                   reference_temperature=0.2),
                       True, list(pb.HEATED3D_BCS), (3, 0.0)),
    lambda: pb.Problem(pb.box_mesh(3, 3, 2, 2, amp=0.1, seed=4),
                       pb.Material(density=5.0, viscosity_model=pb.VISC_CARREAU, mu0=1.0,
                                   mu_inf=0.01, lam=1.0, aexp=2.0, nexp=0.5),
                       False, [b for b in pb.HEATED3D_BCS if b[0] != pb.VAR_T], (0, 0.0)),
    lambda: pb.Problem(pb.box_mesh(3, 2, 3, 2, 1.2, 0.8, 1.0, amp=0.12, seed=6),
                       pb.Material(density=3.0, viscosity=0.7,
                                   momentum_source=(0.5, -2.0, 1.0)),
                       False, [b for b in pb.HEATED3D_BCS if b[0] != pb.VAR_T], (1, 0.3)),
    lambda: pb.Problem(pb.box_mesh(3, 3, 2, 3, 1.0, 0.6, 1.4, amp=0.1, seed=9),
                       pb.Material(density=1.7, viscosity=0.4, heat_capacity=2.2,
                                   conductivity=0.35, momentum_source=(0.0, 0.0, -4.0)),
                       True, list(pb.HEATED3D_BCS), (2, -0.1)),
], ids=["bouss3d", "carreau_t3d", "carreau_ns3d", "newt_ns3d_pert", "newt_t3d_const_src"])
@pytest.mark.parametrize("path", [2, 3, 4])
def test_3d_element_kernels_agree(prob_fn, path):
    """3-D residuals and Jacobians of the other element kernels (path 2: DMMA
    with per-fragment coefficients; path 3: DMMA products over operand
    tables; path 4: sum factorisation -- paths 3 and 4 take Newtonian
    problems and hand Carreau ones to the scalar kernel) equal the
    scalar-FP64 kernel's within 1e-12 (row-scaled), and all equal the oracle.
    Under paths 3 and 4 a residual-only assembly gives the same R bit for
    bit."""
    prob = prob_fn()
    o = oracle.Oracle(prob)
    gn = GomaNewton(prob)
    x = _random_state(o, 23)
    gn.set_assembly_path(path)
    R_tc, a_tc = gn.matrix_fill_full(x)
    R_res, _ = gn.matrix_fill_full(x, jacobian=False)
    gn.set_assembly_path(1)
    R_sc, a_sc = gn.matrix_fill_full(x)
    Ro, ao, _ = o.matrix_fill(x)
    ija = o.ija()
    assert gc.msr_row_scaled_error(ija, a_tc, a_sc) < TOL
    assert gc.msr_row_scaled_error(ija, a_tc, ao) < TOL
    assert np.abs(R_tc - Ro).max() <= TOL * np.abs(Ro).max()
    assert np.abs(R_tc - R_sc).max() <= TOL * np.abs(Ro).max()
    if path in (3, 4):
        assert np.array_equal(R_res, R_tc)


@pytest.mark.parametrize("name", gc.names("assemble", compact=True))
def test_gpu_assembly_matches_reference_at_benchmark_size(name):
    """The 32 x 32 lid-driven cavity at the benchmark size: the whole pattern
    (hash), every residual entry and a seeded sample of Jacobian rows of the
    reference's own assembly."""
    g, case = gc.load(name)
    gn = GomaNewton(gc.problem_from_case(case))
    R, a = gn.matrix_fill_full(g["x"])
    jerr, rerr = gc.compact_rows_check(g, gn.msr_pattern(), a, R)
    assert jerr < TOL and rerr <= TOL


def test_gpu_assembly_matches_oracle_on_the_32_cube():
    """The benchmark workload itself: the 32^3 HEX27 Boussinesq cube
    (1,229,572 unknowns, 308 M nonzeros), every residual entry and every
    Jacobian entry against the oracle's assembly (colour-parallel on the
    host cores), so every colour's persistent element loop runs its full
    4,096 elements."""
    import os
    prob = pb.boussinesq_cube_3d(32, 1e5, 0.71)
    o = oracle.Oracle(prob)
    x = o.dirichlet_init(np.random.default_rng(23).uniform(-1.0, 1.0, o.N))
    pf = oracle.ParallelFill(o, os.cpu_count() or 1)
    try:
        assert pf(x) == 0
        Ro, ao = pf.R, pf.a
        gn = GomaNewton(prob)
        ija = o.ija()
        assert np.array_equal(gn.msr_pattern(), ija)
        R, a = gn.matrix_fill_full(x)
        assert gc.msr_row_scaled_error_fast(ija, a, ao) < TOL
        assert np.abs(R - Ro).max() <= TOL * np.abs(Ro).max()
    finally:
        pf.close()


def test_gpu_reacting_channel_rows_beyond_32bit_offsets_match_oracle():
    """The 64 x 64 x 32 reacting channel (7.0 M unknowns, 2.6e9 nonzeros:
    CSR offsets past 2^31, which the reference's 32-bit MSR cannot hold).
    Rows whose CSR start lies beyond 2^31 -- the last row, the first row
    past the boundary, a pressure row and seeded random ones -- against the
    oracle's element-level assembly of the elements around the row's node,
    and the residual entries of those rows."""
    import ctypes

    import torch
    prob = pb.reacting_channel_3d(64, 64, 32, seed=0)
    gn = GomaNewton(prob)
    assert gn.nnz > 2 ** 31
    x = gn.dirichlet_init(np.random.default_rng(5).uniform(0.5, 1.5, gn.N))
    dx = torch.tensor(x, dtype=torch.float64, device="cuda")
    dR = torch.empty(gn.N, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    gn.matrix_fill_full_device(dx.data_ptr(), dR.data_ptr(), gn.d_vals)
    gn.status()
    R = dR.cpu().numpy()
    fu = np.empty(prob.mesh.num_nodes + 1, np.int32)
    from goma_gb300 import _lib
    _lib.check(gn._L.gb_first_unknown(gn.h, fu.ctypes.data_as(ctypes.POINTER(ctypes.c_int))))
    # first row whose CSR start is past 2^31 (starts ascend)
    lo, hi = 0, gn.N - 1
    while lo < hi:
        mid = (lo + hi) // 2
        if _row_start(gn, mid) >= 2 ** 31:
            hi = mid
        else:
            lo = mid + 1
    r0 = lo
    assert _row_start(gn, r0) >= 2 ** 31 > _row_start(gn, r0 - 1)
    conn = np.asarray(prob.mesh.conn)
    centroids = conn[:, 20]
    nvn = 6
    p_rows = fu[centroids] + nvn
    rows = {r0, gn.N - 1, int(p_rows[p_rows >= r0][0])}
    rows |= set(np.random.default_rng(9).integers(r0, gn.N, 6).tolist())
    o = oracle.Oracle(prob)
    for r in sorted(rows):
        start, cols, vals = gn.csr_row(gn.d_vals, r)
        assert start >= 2 ** 31
        node = int(np.searchsorted(fu, r, side="right") - 1)
        els = np.flatnonzero((conn == node).any(axis=1))
        exp, Rr, Rabs = {}, 0.0, 0.0
        for e in els:
            Re, Je, g, st = o.element(int(e), x)
            assert st == 0
            lr = int(np.flatnonzero(g == r)[0])
            Rr += Re[lr]
            Rabs += abs(Re[lr])
            for c, v in zip(g, Je[lr]):
                exp[int(c)] = exp.get(int(c), 0.0) + v
        ref = np.array([exp.get(int(c), 0.0) for c in cols])
        missing = [c for c, v in exp.items() if v != 0.0 and c not in set(cols.tolist())]
        assert not missing, (r, missing[:5])
        assert np.abs(vals - ref).max() <= TOL * np.abs(ref).max(), r
        assert abs(R[r] - Rr) <= TOL * max(Rabs, 1e-300), r
    del dx, dR
    gn.close()
    torch.cuda.empty_cache()


def _row_start(gn, row):
    import ctypes
    s = ctypes.c_longlong()
    gn._L.gb_csr_row(gn.h, None, int(row), ctypes.byref(s), None, None, 0)
    return s.value
