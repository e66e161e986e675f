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
