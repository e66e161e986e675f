"""Build the problems of the golden cases (tests/golden/*.npz) with the
package's own problem description, so every consumer compares like with
like."""
import json
import os

import numpy as np

from goma_gb300 import problem as pb

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def names(mode=None, compact=False, transient=False):
    """Golden case names (of one mode: assemble, solve, transient);
    compact=True lists the compact records of large cases (sampled Jacobian
    rows, pattern hash) instead of the full ones; transient=True the
    assemblies with time-derivative terms instead of the steady ones."""
    out = []
    for f in sorted(os.listdir(GOLDEN)):
        if f.endswith(".npz"):
            n = f[:-4]
            case = load(n)[1]
            if mode is None and case["mode"] == "transient" and not transient:
                continue
            if ((mode is None or case["mode"] == mode) and bool(case.get("compact")) == compact
                    and bool(case.get("transient")) == (transient or case["mode"] == "transient")):
                out.append(n)
    return out


def compact_rows_check(g, ija, a, R):
    """Row-scaled error of the sampled Jacobian rows and of R of a compact
    record against an assembly (MSR ija / a, residual R), after checking the
    pattern's hash."""
    import hashlib
    n = int(g["N"])
    assert R.size == n and int(ija[n]) == int(g["msr_len"])
    assert hashlib.sha256(np.asarray(ija, "<i4").tobytes()).hexdigest() == str(g["ija_sha256"])
    worst = 0.0
    rows, ptr, cols, vals = g["rows"], g["row_ptr"], g["row_cols"], g["row_vals"]
    for k, i in enumerate(rows):
        c = cols[ptr[k]:ptr[k + 1]]
        v = vals[ptr[k]:ptr[k + 1]]
        assert c[0] == i and np.array_equal(c[1:], ija[ija[i]:ija[i + 1]])
        got = np.concatenate([[a[i]], a[ija[i]:ija[i + 1]]])
        worst = max(worst, np.abs(got - v).max() / max(np.abs(v).max(), 1e-300))
    rerr = np.abs(R - g["R"]).max() / np.abs(g["R"]).max()
    return worst, rerr


def load(name):
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    return g, json.loads(str(g["case"]))


def problem_from_case(case):
    mesh = pb.mesh_from_spec(case["mesh"])
    v = case["visc"]
    if v[0] == "newtonian":
        mat = pb.Material(density=case["rho"], viscosity=v[1])
    else:
        mat = pb.Material(density=case["rho"], viscosity_model=pb.VISC_CARREAU, mu0=v[1],
                          mu_inf=v[2], lam=v[3], aexp=v[4], nexp=v[5])
    energy = case["phys"] in ("nst", "nsty")
    if energy:
        mat.momentum_source_model = pb.SOURCE_BOUSSINESQ
        mat.momentum_source = (0.0, 0.0, -case["ra_pr"])
        mat.volume_expansion = 1.0
        mat.reference_temperature = 0.5
        mat.heat_capacity = 1.0
        mat.conductivity = 1.0
    ns = case.get("nspec", 0)
    if ns:
        # Arrhenius S_w = nu_w k0 exp(-E/T) Y_0, nu = -1 for species 0, +1 after
        k0, E = case["arrhenius"]
        mat.diffusivity = tuple(case["diff"])
        mat.species_source = tuple((pb.SPECIES_SOURCE_ARRHENIUS, (k0, E, -1.0 if w == 0 else 1.0, 0))
                                   for w in range(ns))
    if "heat" in case:
        mat.heat_source_model = pb.HEAT_SOURCE_EXPONENTIAL
        mat.heat_source = tuple(case["heat"])
    U1, U2, U3, T = pb.VAR_U1, pb.VAR_U2, pb.VAR_U3, pb.VAR_T
    bcs = {"cavity2d": pb.CAVITY2D_BCS, "bfs2d": pb.BFS2D_BCS,
           "cube_heated": pb.HEATED3D_BCS, "cube_species": pb.SPECIES3D_BCS,
           "bratu2d": pb.bratu_square_2d(1).bcs,
           "channel2d_t": [(U1, 1, 0.0), (U2, 1, 0.0), (U1, 3, 0.0), (U2, 3, 0.0),
                           (U1, 4, 1.0), (U2, 4, 0.0), (T, 4, 1.0)],
           "box_open_top": [(c, s, 0.0) for s in (1, 2, 3, 4, 5) for c in (U1, U2, U3)]
           + [(T, 1, 1.0)]}[case["bc"]]
    kinds = {"QSIDE": pb.IBC_QSIDE, "QCONV": pb.IBC_QCONV, "FLOW_PRESSURE": pb.IBC_FLOW_PRESSURE}
    ibcs = [(kinds[name], ss, float(vals[0]), float(vals[1]) if len(vals) > 1 else 0.0)
            for name, ss, vals in case.get("ibc", [])]
    return pb.Problem(mesh, mat, energy, list(bcs), (0, 0.0) if case["datum"] else (-1, 0.0),
                      num_species=ns, ibcs=ibcs)


def msr_row_scaled_error(ija, a, ref):
    """max over rows of max_j |a_ij - ref_ij| / max_j |ref_ij| (MSR)."""
    N = ija[0] - 1
    worst = 0.0
    for i in range(N):
        lo, hi = ija[i], ija[i + 1]
        scale = max(abs(ref[i]), np.abs(ref[lo:hi]).max() if hi > lo else 0.0, 1e-300)
        d = max(abs(a[i] - ref[i]), np.abs(a[lo:hi] - ref[lo:hi]).max() if hi > lo else 0.0)
        worst = max(worst, d / scale)
    return worst


def msr_row_scaled_error_fast(ija, a, ref):
    """msr_row_scaled_error, vectorised for large matrices (every row must
    have off-diagonal entries)."""
    N = int(ija[0]) - 1
    lens = np.diff(np.asarray(ija[:N + 1], np.int64))
    assert (lens > 0).all()
    starts = np.asarray(ija[:N], np.int64) - (N + 1)
    dm = np.maximum.reduceat(np.abs(a[N + 1:] - ref[N + 1:]), starts)
    rm = np.maximum.reduceat(np.abs(ref[N + 1:]), starts)
    dm = np.maximum(dm, np.abs(a[:N] - ref[:N]))
    rm = np.maximum(rm, np.abs(ref[:N]))
    return float((dm / np.maximum(rm, 1e-300)).max())
