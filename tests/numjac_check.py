"""The reference's analytic-Jacobian checker, restated for the tests.

numerical_jacobian (src/mm_numjac.c:716-1466), in its default bracketed
form with Debug_Flag = -2 (rows scaled by their row sums,
row_sum_scaling_scale src/sl_matrix_util.c:441), steady case:

- assemble R and J at x; scale the rows (scale_i = sign(a_ii) sum_j |a_ij|);
- x_scale per variable type: the RMS of x over the unknowns of that type, 1
  where that is zero (:862-895);
- for every column j: dx = x_scale(type j) * FD_DELTA_UNKNOWN (1e-6,
  include/mm_numjac.h:50), x1 = x + dx e_j, assemble R1 and J1 at x1 and
  scale their rows by the same scale vector (:1003-1188);
- for every unknown i on the nodes of the elements that contain j's node
  (:1063-1090): with aj = J(i, j), aj_1 = J1(i, j), the perturbed residual
  must lie in [R_i + dx min(aj, aj_1), R_i + dx max(aj, aj_1)] widened by
  roundoff * resid_scale on each side, roundoff = 1e-11 and resid_scale =
  max(|R_i|, |J1(i, k)| x_scale(type k) over the row) (:1258-1300); an
  entry outside is flagged (:1301-1349).  Pairs the interaction mask leaves
  out (energy equation, pressure unknown) are flagged when either Jacobian
  holds a value there or R1_i moves by more than the roundoff band
  (:1410-1433).

With the checker on (Debug_Flag < 0) the reference assembles the bare
equations: put_dirichlet_in_matrix returns at once (src/bc_dirich.c:73-74),
which also leaves out the pressure datum.  without_dirichlet() gives the
same problem without its Dirichlet cards and datum for the fills.

Matrices are handled dense (these are small problems)."""
import dataclasses

import numpy as np


def without_dirichlet(prob):
    return dataclasses.replace(prob, bcs=[], pressure_datum=(-1, 0.0))


FD_DELTA_UNKNOWN = 1e-6
ROUNDOFF = 1e-11


def msr_to_dense(ija, a):
    N = int(ija[0]) - 1
    A = np.zeros((N, N))
    A[np.arange(N), np.arange(N)] = a[:N]
    for i in range(N):
        A[i, ija[ija[i]:ija[i + 1]]] = a[ija[i]:ija[i + 1]]
    return A


def row_sum_scale(A, R):
    s = np.abs(A).sum(axis=1)
    d = np.diag(A)
    s = np.where(np.abs(d) > 1e-200, np.where(d < 0, -s, s), s)
    s = np.where(s == 0.0, 1.0, s)
    return A / s[:, None], R / s, s


class Layout:
    """Per-unknown variable type and node, and the element lists the
    checker needs, from a problem and its first-unknown map."""

    def __init__(self, prob, fu):
        self.fu = np.asarray(fu)
        dim = prob.dim
        nvn = dim + (1 if prob.energy else 0) + prob.num_species
        N = int(self.fu[-1])
        self.node = np.searchsorted(self.fu, np.arange(N), side="right") - 1
        off = np.arange(N) - self.fu[self.node]
        # variable types: velocity components 0..dim-1, temperature, one
        # type for all species, pressure
        typ = np.where(off < dim, off, 0)
        if prob.energy:
            typ = np.where(off == dim, 10, typ)
        typ = np.where((off >= dim + (1 if prob.energy else 0)) & (off < nvn), 20, typ)
        typ = np.where(off >= nvn, 30, typ)
        self.type = typ
        self.is_T = (off == dim) if prob.energy else np.zeros(N, bool)
        self.is_P = off >= nvn
        conn = np.asarray(prob.mesh.conn)
        self.conn = conn
        nnodes = prob.mesh.num_nodes
        self.node_elems = [[] for _ in range(nnodes)]
        for e, row in enumerate(conn):
            for n in row:
                self.node_elems[n].append(e)
        self.unknowns_of_node = [np.arange(self.fu[n], self.fu[n + 1]) for n in range(nnodes)]


def check(layout, fill, x):
    """Runs the checker; fill(x) -> (R, dense J).  Returns the flagged
    entries as (kind, i, j) tuples."""
    x = np.asarray(x, np.float64)
    R0, A0 = fill(x)
    A, R, scale = row_sum_scale(A0, R0)
    types = np.unique(layout.type)
    xs = {}
    for t in types:
        v = np.sqrt(np.mean(x[layout.type == t] ** 2))
        xs[t] = v if v != 0.0 else 1.0
    xsc = np.array([xs[t] for t in layout.type])
    flagged = []
    N = x.size
    for j in range(N):
        dx = xsc[j] * FD_DELTA_UNKNOWN
        x1 = x.copy()
        x1[j] = x[j] + dx
        R1u, A1u = fill(x1)
        A1 = A1u / scale[:, None]
        R1 = R1u / scale
        nodes = set()
        for e in layout.node_elems[layout.node[j]]:
            nodes.update(layout.conn[e].tolist())
        dofs = np.concatenate([layout.unknowns_of_node[n] for n in sorted(nodes)])
        for i in dofs:
            aj, aj1 = A[i, j], A1[i, j]
            lo, hi = sorted((dx * aj, dx * aj1))
            rs = max(abs(R[i]), np.max(np.abs(A1[i]) * xsc))
            masked = layout.is_T[i] and layout.is_P[j]
            if masked:
                if aj != 0.0 or aj1 != 0.0:
                    flagged.append(("mask_analytic", int(i), int(j)))
                if abs(R1[i] - R[i]) > ROUNDOFF * rs:
                    flagged.append(("mask_numerical", int(i), int(j)))
                continue
            if R1[i] < R[i] + lo - ROUNDOFF * rs or R1[i] > R[i] + hi + ROUNDOFF * rs:
                flagged.append(("bracket", int(i), int(j)))
    return flagged
