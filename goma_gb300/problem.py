"""Problem description for the Q2/P1 Newton path: structured meshes,
material, Dirichlet cards, and the ctypes mirror of ``gb_problem_desc``
(include/gb_problem.h).

The fields mirror what the reference reads from its input deck, material
file and Exodus mesh (see the header).  Structured box meshes use the
Exodus/Goma QUAD9 and HEX27 local node order (src/rf_shape.c:361, :1105).
"""
import ctypes
from dataclasses import dataclass, field
from typing import List, Tuple

import numpy as np

VAR_U1, VAR_U2, VAR_U3, VAR_T, VAR_P = 0, 1, 2, 3, 9
VISC_NEWTONIAN, VISC_CARREAU = 0, 1
SOURCE_CONSTANT, SOURCE_BOUSSINESQ = 0, 1
MAX_SPECIES = 4
SPECIES_SOURCE_NONE, SPECIES_SOURCE_CONSTANT, SPECIES_SOURCE_ARRHENIUS = 0, 1, 2
HEAT_SOURCE_NONE, HEAT_SOURCE_CONSTANT, HEAT_SOURCE_EXPONENTIAL = 0, 1, 2
IBC_QSIDE, IBC_QCONV, IBC_FLOW_PRESSURE = 1, 2, 3


def VAR_Y(w):
    """Variable id of species w (GB_VAR_Y in include/gb_problem.h)."""
    return 100 + w

# grid offsets (0..2) of the local nodes, Goma order
QUAD9_LOCAL = np.array([[0, 0], [2, 0], [2, 2], [0, 2], [1, 0], [2, 1], [1, 2], [0, 1], [1, 1]])
HEX27_LOCAL = np.array([
    [0, 0, 0], [2, 0, 0], [2, 2, 0], [0, 2, 0], [0, 0, 2], [2, 0, 2], [2, 2, 2], [0, 2, 2],
    [1, 0, 0], [2, 1, 0], [1, 2, 0], [0, 1, 0], [0, 0, 1], [2, 0, 1], [2, 2, 1], [0, 2, 1],
    [1, 0, 2], [2, 1, 2], [1, 2, 2], [0, 1, 2], [1, 1, 1], [1, 1, 0], [1, 1, 2], [0, 1, 1],
    [2, 1, 1], [1, 0, 1], [1, 2, 1]])

_M64 = (1 << 64) - 1


def _mix64(z):
    """splitmix64 finaliser on a uint64 array (fixed integer hash)."""
    with np.errstate(over="ignore"):
        z = z + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def jitter(seed, nodes, axis):
    """Uniform(-1, 1) per (seed, node, axis) from the fixed hash."""
    with np.errstate(over="ignore"):
        z = (np.uint64(seed) * np.uint64(0x100000001B3) + nodes.astype(np.uint64) * np.uint64(3)
             + np.uint64(axis))
    h = _mix64(z)
    return (h >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0) * 2.0 - 1.0


@dataclass
class Mesh:
    dim: int
    coords: np.ndarray      # (num_nodes, dim) float64
    conn: np.ndarray        # (num_elems, 9|27) int32
    node_sets: List[np.ndarray]  # node set id k+1 -> ascending node ids
    shape: Tuple[int, ...] = ()
    # side set id k+1 -> (elements, Exodus side numbers), both int32
    side_sets: List[Tuple[np.ndarray, np.ndarray]] = field(default_factory=list)

    @property
    def num_nodes(self):
        return self.coords.shape[0]

    @property
    def num_elems(self):
        return self.conn.shape[0]


def box_mesh(dim, nx, ny, nz=1, lx=1.0, ly=1.0, lz=1.0, amp=0.0, seed=0):
    """Structured QUAD9 (dim 2) or HEX27 (dim 3) box.

    Nodes are numbered x fastest over the (2nx+1) x (2ny+1) [x (2nz+1)]
    grid, elements x fastest.  With amp > 0 every strictly interior node
    moves by amp * spacing * U(-1,1) per axis (fixed hash of seed, node,
    axis).  Node sets: 2-D 1 y=0, 2 x=Lx, 3 y=Ly, 4 x=0, 5 x=0 & y<=Ly/2,
    6 x=0 & y>=Ly/2; 3-D 1 x=0, 2 x=Lx, 3 y=0, 4 y=Ly, 5 z=0, 6 z=Lz.
    """
    NX, NY = 2 * nx + 1, 2 * ny + 1
    NZ = 2 * nz + 1 if dim == 3 else 1
    k, j, i = np.meshgrid(np.arange(NZ), np.arange(NY), np.arange(NX), indexing="ij")
    i, j, k = i.ravel(), j.ravel(), k.ravel()
    nid = np.arange(i.size, dtype=np.int64)
    x = lx * i / (NX - 1)
    y = ly * j / (NY - 1)
    cols = [x, y]
    if dim == 3:
        cols.append(lz * k / (NZ - 1))
    if amp != 0.0:
        inner = (i > 0) & (i < NX - 1) & (j > 0) & (j < NY - 1)
        if dim == 3:
            inner &= (k > 0) & (k < NZ - 1)
        ext = [lx, ly, lz]
        npts = [NX, NY, NZ]
        for ax in range(dim):
            d = amp * (ext[ax] / (npts[ax] - 1)) * jitter(seed, nid, ax)
            cols[ax] = np.where(inner, cols[ax] + d, cols[ax])
    coords = np.stack(cols, axis=1).astype(np.float64)
    if dim == 2:
        ey, ex = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")
        ex, ey = ex.ravel(), ey.ravel()
        gi = 2 * ex[:, None] + QUAD9_LOCAL[None, :, 0]
        gj = 2 * ey[:, None] + QUAD9_LOCAL[None, :, 1]
        conn = gi + NX * gj
        sets = [j == 0, i == NX - 1, j == NY - 1, i == 0, (i == 0) & (2 * j <= NY - 1),
                (i == 0) & (2 * j >= NY - 1)]
    else:
        ez, ey, ex = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
        ex, ey, ez = ex.ravel(), ey.ravel(), ez.ravel()
        gi = 2 * ex[:, None] + HEX27_LOCAL[None, :, 0]
        gj = 2 * ey[:, None] + HEX27_LOCAL[None, :, 1]
        gk = 2 * ez[:, None] + HEX27_LOCAL[None, :, 2]
        conn = gi + NX * (gj + NY * gk)
        sets = [i == 0, i == NX - 1, j == 0, j == NY - 1, k == 0, k == NZ - 1]
    node_sets = [np.nonzero(s)[0].astype(np.int32) for s in sets]
    shape = (nx, ny) if dim == 2 else (nx, ny, nz)
    # side sets on the same boundaries as node sets 1..4 (2-D) / 1..6 (3-D),
    # Exodus side numbers: QUAD9 1 t=-1, 2 s=+1, 3 t=+1, 4 s=-1; HEX27 the
    # same and 5 u=-1, 6 u=+1
    eid = np.arange(nx * ny * (nz if dim == 3 else 1), dtype=np.int32)
    if dim == 2:
        sel = [(ey == 0, 1), (ex == nx - 1, 2), (ey == ny - 1, 3), (ex == 0, 4)]
    else:
        sel = [(ex == 0, 4), (ex == nx - 1, 2), (ey == 0, 1), (ey == ny - 1, 3), (ez == 0, 5),
               (ez == nz - 1, 6)]
    side_sets = [(eid[m], np.full(int(m.sum()), sd, np.int32)) for m, sd in sel]
    return Mesh(dim, coords, np.ascontiguousarray(conn, dtype=np.int32), node_sets, shape,
                side_sets)


def mesh_from_spec(spec):
    """Parse 'quad9 NX NY LX LY [AMP SEED]' or 'hex27 NX NY NZ LX LY LZ [AMP SEED]'."""
    t = spec.split()
    if t[0] == "quad9":
        nx, ny = int(t[1]), int(t[2])
        lx, ly = float(t[3]), float(t[4])
        amp, seed = (float(t[5]), int(t[6])) if len(t) > 5 else (0.0, 0)
        return box_mesh(2, nx, ny, 1, lx, ly, 0.0, amp, seed)
    if t[0] == "hex27":
        nx, ny, nz = int(t[1]), int(t[2]), int(t[3])
        lx, ly, lz = float(t[4]), float(t[5]), float(t[6])
        amp, seed = (float(t[7]), int(t[8])) if len(t) > 7 else (0.0, 0)
        return box_mesh(3, nx, ny, nz, lx, ly, lz, amp, seed)
    raise ValueError("unknown mesh spec %r" % spec)


@dataclass
class Material:
    density: float = 1.0
    viscosity_model: int = VISC_NEWTONIAN
    viscosity: float = 1.0
    mu0: float = 1.0
    mu_inf: float = 0.0
    lam: float = 1.0
    aexp: float = 2.0
    nexp: float = 1.0
    heat_capacity: float = 1.0
    conductivity: float = 1.0
    momentum_source_model: int = SOURCE_CONSTANT
    momentum_source: Tuple[float, float, float] = (0.0, 0.0, 0.0)
    volume_expansion: float = 0.0
    reference_temperature: float = 0.0
    # species w: Fickian diffusivity and source; a source is (model, params),
    # params (S,) for CONSTANT, (k0, E, nu, s) for ARRHENIUS:
    # S_w = nu k0 exp(-E/T) Y_s
    diffusivity: Tuple[float, ...] = ()
    species_source: Tuple[Tuple[int, Tuple[float, ...]], ...] = ()
    # energy equation heat source: HEAT_SOURCE_CONSTANT h = c0, or
    # HEAT_SOURCE_EXPONENTIAL h = c0 exp(c1 T) (Frank-Kamenetskii / Bratu)
    heat_source_model: int = HEAT_SOURCE_NONE
    heat_source: Tuple[float, float] = (0.0, 0.0)


@dataclass
class Problem:
    mesh: Mesh
    material: Material
    energy: bool = False
    # Dirichlet cards in deck order: (variable, node set id (1-based), value)
    bcs: List[Tuple[int, int, float]] = field(default_factory=list)
    pressure_datum: Tuple[int, float] = (-1, 0.0)
    num_species: int = 0
    # integrated boundary conditions: (IBC_* type, side set id (1-based),
    # value 0, value 1)
    ibcs: List[Tuple[int, int, float, float]] = field(default_factory=list)

    @property
    def dim(self):
        return self.mesh.dim


class CMaterial(ctypes.Structure):
    _fields_ = [("density", ctypes.c_double), ("viscosity_model", ctypes.c_int),
                ("viscosity", ctypes.c_double), ("mu0", ctypes.c_double),
                ("mu_inf", ctypes.c_double), ("lambda_", ctypes.c_double),
                ("aexp", ctypes.c_double), ("nexp", ctypes.c_double),
                ("heat_capacity", ctypes.c_double), ("conductivity", ctypes.c_double),
                ("momentum_source_model", ctypes.c_int),
                ("momentum_source", ctypes.c_double * 3),
                ("volume_expansion", ctypes.c_double),
                ("reference_temperature", ctypes.c_double),
                ("diffusivity", ctypes.c_double * MAX_SPECIES),
                ("species_source_model", ctypes.c_int * MAX_SPECIES),
                ("species_source", (ctypes.c_double * 4) * MAX_SPECIES),
                ("heat_source_model", ctypes.c_int), ("heat_source", ctypes.c_double * 2)]


class CProblemDesc(ctypes.Structure):
    _fields_ = [("dim", ctypes.c_int), ("num_nodes", ctypes.c_int), ("num_elems", ctypes.c_int),
                ("coords", ctypes.POINTER(ctypes.c_double)),
                ("conn", ctypes.POINTER(ctypes.c_int)), ("energy", ctypes.c_int),
                ("num_species", ctypes.c_int), ("mat", CMaterial), ("num_bc", ctypes.c_int),
                ("bc_var", ctypes.POINTER(ctypes.c_int)),
                ("bc_value", ctypes.POINTER(ctypes.c_double)),
                ("bc_ptr", ctypes.POINTER(ctypes.c_int)),
                ("bc_nodes", ctypes.POINTER(ctypes.c_int)),
                ("pressure_datum_elem", ctypes.c_int),
                ("pressure_datum_value", ctypes.c_double),
                ("num_ibc", ctypes.c_int), ("ibc_type", ctypes.POINTER(ctypes.c_int)),
                ("ibc_value", ctypes.POINTER(ctypes.c_double)),
                ("ibc_ptr", ctypes.POINTER(ctypes.c_int)),
                ("ibc_elem", ctypes.POINTER(ctypes.c_int)),
                ("ibc_side", ctypes.POINTER(ctypes.c_int))]


def c_material(mt: Material):
    cm = CMaterial(mt.density, mt.viscosity_model, mt.viscosity, mt.mu0, mt.mu_inf, mt.lam,
                   mt.aexp, mt.nexp, mt.heat_capacity, mt.conductivity,
                   mt.momentum_source_model, (ctypes.c_double * 3)(*mt.momentum_source),
                   mt.volume_expansion, mt.reference_temperature)
    for w, d in enumerate(mt.diffusivity):
        cm.diffusivity[w] = d
    for w, (model, params) in enumerate(mt.species_source):
        cm.species_source_model[w] = model
        for k, v in enumerate(params):
            cm.species_source[w][k] = v
    cm.heat_source_model = mt.heat_source_model
    cm.heat_source[0], cm.heat_source[1] = mt.heat_source
    return cm


def make_desc(prob: Problem):
    """Build the C description; returns (desc, keepalive) -- keep the second
    object alive while the description is in use."""
    m = prob.mesh
    coords = np.ascontiguousarray(m.coords, dtype=np.float64)
    conn = np.ascontiguousarray(m.conn, dtype=np.int32)
    bc_var = np.array([b[0] for b in prob.bcs], dtype=np.int32)
    bc_val = np.array([b[2] for b in prob.bcs], dtype=np.float64)
    lists = [m.node_sets[b[1] - 1] for b in prob.bcs]
    bc_ptr = np.zeros(len(lists) + 1, dtype=np.int32)
    bc_ptr[1:] = np.cumsum([len(l) for l in lists]) if lists else []
    bc_nodes = (np.concatenate(lists).astype(np.int32) if lists else np.zeros(1, np.int32))
    if bc_var.size == 0:
        bc_var = np.zeros(1, np.int32)
        bc_val = np.zeros(1, np.float64)
    cm = c_material(prob.material)
    P = lambda a, t: a.ctypes.data_as(ctypes.POINTER(t))  # noqa: E731
    ib_type = np.array([b[0] for b in prob.ibcs] or [0], dtype=np.int32)
    ib_val = np.array([v for b in prob.ibcs for v in (b[2], b[3])] or [0.0], dtype=np.float64)
    ib_sets = [m.side_sets[b[1] - 1] for b in prob.ibcs]
    ib_ptr = np.zeros(len(ib_sets) + 1, dtype=np.int32)
    ib_ptr[1:] = np.cumsum([len(e) for e, _ in ib_sets]) if ib_sets else []
    ib_elem = (np.concatenate([e for e, _ in ib_sets]).astype(np.int32) if ib_sets
               else np.zeros(1, np.int32))
    ib_side = (np.concatenate([sd for _, sd in ib_sets]).astype(np.int32) if ib_sets
               else np.zeros(1, np.int32))
    d = CProblemDesc(m.dim, m.num_nodes, m.num_elems, P(coords, ctypes.c_double),
                     P(conn, ctypes.c_int), 1 if prob.energy else 0, int(prob.num_species),
                     cm, len(prob.bcs),
                     P(bc_var, ctypes.c_int), P(bc_val, ctypes.c_double), P(bc_ptr, ctypes.c_int),
                     P(bc_nodes, ctypes.c_int), int(prob.pressure_datum[0]),
                     float(prob.pressure_datum[1]), len(prob.ibcs), P(ib_type, ctypes.c_int),
                     P(ib_val, ctypes.c_double), P(ib_ptr, ctypes.c_int),
                     P(ib_elem, ctypes.c_int), P(ib_side, ctypes.c_int))
    return d, (coords, conn, bc_var, bc_val, bc_ptr, bc_nodes, ib_type, ib_val, ib_ptr, ib_elem,
               ib_side)


# ------------------------------------------------------------ standard cases

CAVITY2D_BCS = [(VAR_U1, 1, 0.0), (VAR_U2, 1, 0.0), (VAR_U1, 2, 0.0), (VAR_U2, 2, 0.0),
                (VAR_U1, 4, 0.0), (VAR_U2, 4, 0.0), (VAR_U1, 3, 1.0), (VAR_U2, 3, 0.0)]
BFS2D_BCS = [(VAR_U1, 1, 0.0), (VAR_U2, 1, 0.0), (VAR_U1, 3, 0.0), (VAR_U2, 3, 0.0),
             (VAR_U1, 5, 0.0), (VAR_U2, 5, 0.0), (VAR_U1, 6, 1.0), (VAR_U2, 6, 0.0)]
HEATED3D_BCS = ([(c, s, 0.0) for s in (1, 2, 3, 4, 5, 6) for c in (VAR_U1, VAR_U2, VAR_U3)]
                + [(VAR_T, 1, 1.0), (VAR_T, 2, 0.0)])
# heated box fed with species 0 at x = 0; T in [1, 2] keeps exp(-E/T) finite
SPECIES3D_BCS = ([(c, s, 0.0) for s in (1, 2, 3, 4, 5, 6) for c in (VAR_U1, VAR_U2, VAR_U3)]
                 + [(VAR_T, 1, 2.0), (VAR_T, 2, 1.0), (VAR_Y(0), 1, 1.0), (VAR_Y(1), 1, 0.0)])


def lid_cavity_2d(n, re=100.0, mesh=None):
    """Unit-square lid-driven cavity, n x n QUAD9, mu = 1, rho = Re."""
    mesh = mesh or box_mesh(2, n, n)
    return Problem(mesh, Material(density=re, viscosity=1.0), False, list(CAVITY2D_BCS), (0, 0.0))


def boussinesq_cube_3d(n, ra=1e5, pr=0.71, mesh=None):
    """Unit-cube natural convection, n^3 HEX27: rho = Cp = k = 1, mu = Pr,
    gravity -z with g beta = Ra Pr, T = 1 at x = 0, T = 0 at x = 1,
    reference temperature 0.5."""
    mesh = mesh or box_mesh(3, n, n, n)
    mat = Material(density=1.0, viscosity=pr, heat_capacity=1.0, conductivity=1.0,
                   momentum_source_model=SOURCE_BOUSSINESQ,
                   momentum_source=(0.0, 0.0, -ra * pr), volume_expansion=1.0,
                   reference_temperature=0.5)
    return Problem(mesh, mat, True, list(HEATED3D_BCS), (0, 0.0))


# reacting channel: plug inflow at x = 0, no-slip walls y = 0, Ly, z = 0, Lz
# (walls win at the inlet edges), outflow at x = Lx; hot feed of species 0
REACTING3D_BCS = ([(VAR_U1, 1, 1.0), (VAR_U2, 1, 0.0), (VAR_U3, 1, 0.0)]
                  + [(c, s, 0.0) for s in (3, 4, 5, 6) for c in (VAR_U1, VAR_U2, VAR_U3)]
                  + [(VAR_T, 1, 2.0), (VAR_T, 3, 1.0), (VAR_T, 4, 1.0),
                     (VAR_Y(0), 1, 1.0), (VAR_Y(1), 1, 0.0)])


def reacting_channel_3d(nx, ny, nz, lx=2.0, ly=2.0, lz=1.0, seed=0, re=100.0, diffusivity=1e-3,
                        activation=2.0, mesh=None):
    """Channel flow with energy and two dilute species reacting A -> B at an
    Arrhenius rate: HEX27 box [0, Lx] x [0, Ly] x [0, Lz], rho = Cp = 1,
    mu = 1 / Re, k = 1 / Re, Fickian D for both species, source
    S_0 = -k0 exp(-E / T) Y_0, S_1 = +k0 exp(-E / T) Y_0 with the rate
    constant k0 drawn uniformly from [0.1, 10] by `seed`.  The outflow face
    fixes the pressure level, so there is no pressure datum."""
    mesh = mesh or box_mesh(3, nx, ny, nz, lx, ly, lz)
    k0 = float(np.random.default_rng(seed).uniform(0.1, 10.0))
    mat = Material(density=1.0, viscosity=1.0 / re, heat_capacity=1.0, conductivity=1.0 / re,
                   diffusivity=(diffusivity, diffusivity),
                   species_source=((SPECIES_SOURCE_ARRHENIUS, (k0, activation, -1.0, 0.0)),
                                   (SPECIES_SOURCE_ARRHENIUS, (k0, activation, 1.0, 0.0))))
    return Problem(mesh, mat, True, list(REACTING3D_BCS), (-1, 0.0), 2)


def bratu_square_2d(n, lam=1.0, mesh=None):
    """Frank-Kamenetskii / Bratu problem on the unit square, n x n QUAD9: the
    energy equation with the heat source lam exp(T), unit conductivity, T =
    0 on the whole boundary; the fluid is at rest (no-slip walls all round,
    no body force, pressure datum on element 0), so the flow rows have the
    zero solution.  Its solution branch has a fold at lam ~ 6.808."""
    mesh = mesh or box_mesh(2, n, n)
    mat = Material(density=1.0, viscosity=1.0, heat_capacity=1.0, conductivity=1.0,
                   heat_source_model=HEAT_SOURCE_EXPONENTIAL, heat_source=(lam, 1.0))
    bcs = list(CAVITY2D_BCS[:6]) + [(VAR_U1, 3, 0.0), (VAR_U2, 3, 0.0)]
    bcs += [(VAR_T, s, 0.0) for s in (1, 2, 3, 4)]
    return Problem(mesh, mat, True, bcs, (0, 0.0))


def carreau_step_2d(nx, ny, re, lx=3.0, ly=1.0, mesh=None, mu0=1.0, mu_inf=0.01, lam=1.0,
                    aexp=2.0, nexp=0.5):
    """Channel with a plug inlet on the upper half of x = 0 and a wall on
    the lower half (the step face), Carreau-Yasuda fluid, outflow at x = Lx."""
    mesh = mesh or box_mesh(2, nx, ny, 1, lx, ly)
    mat = Material(density=re, viscosity_model=VISC_CARREAU, mu0=mu0, mu_inf=mu_inf, lam=lam,
                   aexp=aexp, nexp=nexp)
    return Problem(mesh, mat, False, list(BFS2D_BCS), (-1, 0.0))


# ------------------------------------------------------------ batches

@dataclass
class BatchMember:
    kind: str          # "cavity" or "channel"
    n: int             # n x n QUAD9 elements on the unit square
    re: float          # Reynolds number (rho = Re, mu = U = L = 1)
    elems: Tuple[int, int]   # element range in the union
    nodes: Tuple[int, int]   # node range in the union


@dataclass
class ProblemBatch:
    problem: Problem            # the disjoint union, material density 1
    elem_re: np.ndarray         # Reynolds number (density) of every element
    members: List[BatchMember]


def _member_bcs(kind, mesh, set_base, node_base):
    """Node sets (global node ids) and Dirichlet cards of one member.  Cavity:
    no-slip walls, lid u = 1 on y = 1, its first element's first pressure
    pinned to 0.  Channel: parabolic inflow u = 4 y (1 - y) on x = 0 (one
    node set per inlet node), no-slip on y = 0 and y = 1 (walls win at the
    inlet corners), natural outflow on x = 1."""
    sets = [s + node_base for s in mesh.node_sets]
    bcs = []
    if kind == "cavity":
        for var, sid, val in CAVITY2D_BCS:
            bcs.append((var, set_base + sid, val))
        sets.append(np.array([node_base + mesh.conn[0, 8]], np.int32))
        bcs.append((VAR_P, set_base + len(sets), 0.0))
    else:
        inlet = mesh.node_sets[3]
        for nd in inlet:
            y = mesh.coords[nd, 1]
            sets.append(np.array([node_base + nd], np.int32))
            bcs.append((VAR_U1, set_base + len(sets), 4.0 * y * (1.0 - y)))
        for sid in (4,):
            bcs.append((VAR_U2, set_base + sid, 0.0))
        for sid in (1, 3):
            bcs.append((VAR_U1, set_base + sid, 0.0))
            bcs.append((VAR_U2, set_base + sid, 0.0))
    return sets, bcs


def batch_shard(num, seed, rank, world, nmin=16, nmax=64):
    """Members of a `num`-problem sweep that rank `rank` of `world` solves:
    the problems are independent, so they are dealt out with no exchange.
    Members go largest first to the rank with the least work so far (the
    work of a member ~ its element count n^2), so the ranks' loads differ by
    at most one member; the same seed gives every rank the same partition."""
    ns = np.random.default_rng(seed).integers(nmin, nmax + 1, num)
    load = [0] * world
    owner = np.empty(num, np.int64)
    for p in sorted(range(num), key=lambda q: (-int(ns[q]), q)):
        r = min(range(world), key=lambda k: (load[k], k))
        owner[p] = r
        load[r] += int(ns[p]) ** 2
    return [p for p in range(num) if owner[p] == rank]


def batch_sweep_2d(num=512, seed=0, nmin=16, nmax=64, re_min=10.0, re_max=1000.0,
                   kinds=("cavity", "channel"), members=None):
    """`num` independent unit-square QUAD9 Q2/P1 problems drawn from `seed`:
    mesh n x n with n uniform in [nmin, nmax], Re log-uniform in
    [re_min, re_max], lid-driven cavity or channel alternately.  Returned as
    one disjoint union (nodes, elements and unknowns of member p follow those
    of member p - 1) with the per-element Reynolds numbers, so that one
    context assembles and solves all of them together.  `members` (a list of
    member indices, e.g. from batch_shard) keeps only those problems, with
    the same draws as the full sweep."""
    rng = np.random.default_rng(seed)
    ns = rng.integers(nmin, nmax + 1, num)
    res = np.exp(rng.uniform(np.log(re_min), np.log(re_max), num))
    chosen = range(num) if members is None else members
    coords, conns, sets, bcs, rho, members = [], [], [], [], [], []
    node_base = elem_base = 0
    for p in chosen:
        kind = kinds[p % len(kinds)]
        m = box_mesh(2, int(ns[p]), int(ns[p]))
        msets, mbcs = _member_bcs(kind, m, len(sets), node_base)
        coords.append(m.coords + np.array([1.5 * p, 0.0]))
        conns.append(m.conn + node_base)
        sets.extend(msets)
        bcs.extend(mbcs)
        rho.append(np.full(m.num_elems, res[p]))
        members.append(BatchMember(kind, int(ns[p]), float(res[p]),
                                   (elem_base, elem_base + m.num_elems),
                                   (node_base, node_base + m.num_nodes)))
        node_base += m.num_nodes
        elem_base += m.num_elems
    mesh = Mesh(2, np.vstack(coords), np.ascontiguousarray(np.vstack(conns), np.int32), sets,
                None)
    prob = Problem(mesh, Material(density=1.0, viscosity=1.0), False, bcs, (-1, 0.0))
    return ProblemBatch(prob, np.concatenate(rho), members)


def batch_member_problem(batch, p):
    """Member p of a batch as a problem of its own."""
    mb = batch.members[p]
    m = box_mesh(2, mb.n, mb.n)
    sets, bcs = _member_bcs(mb.kind, m, 0, 0)
    m.node_sets = sets
    return Problem(m, Material(density=mb.re, viscosity=1.0), False, bcs, (-1, 0.0))
