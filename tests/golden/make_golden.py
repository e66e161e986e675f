"""Generate the golden vectors that pin the CPU oracle to the reference.

Runs the unmodified reference Goma (built by ``oracle/build_ref.sh`` into
``oracle/_ref/goma_ref``) on small seeded cases and stores what its
``matrix_fill_full`` (src/mm_fill.c:158) assembled -- the MSR pattern
``ija``, the MSR values ``a`` and the residual ``R`` -- and, for the
``solve`` cases, the converged Newton solution written by
``write_ascii_soln`` (src/rf_util.c:2387).  Each case is one ``.npz`` file
next to this script.  Test infrastructure only: needs the reference tree,
so it runs in the build container, never on the GPU machine.

    python tests/golden/make_golden.py [--ref /root/reference] [case ...]
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
GOMA = os.path.join(REPO, "oracle", "_ref", "goma_ref")

# ---------------------------------------------------------------- cases
# phys: "ns" (momentum + continuity), "nst" (+ energy, Boussinesq source)
# visc: ("newtonian", mu) or ("carreau", mu0, muinf, lam, aexp, nexp)
CASES = {
    # 2-D lid-driven cavity, seeded state, affine and perturbed elements
    "cav2d_2x2": dict(mesh="quad9 2 2 1 1", phys="ns", rho=100.0, visc=("newtonian", 1.0),
                      bc="cavity2d", datum=True, mode="assemble", seed=1),
    "cav2d_3x2_pert": dict(mesh="quad9 3 2 1.5 1 0.15 7", phys="ns", rho=100.0,
                           visc=("newtonian", 1.0), bc="cavity2d", datum=True,
                           mode="assemble", seed=2),
    # Carreau-Yasuda channel with a plug inlet on the upper half of x = 0
    "bfs2d_4x2_carreau": dict(mesh="quad9 4 2 3 1 0.1 11", phys="ns", rho=50.0,
                              visc=("carreau", 1.0, 0.01, 1.0, 2.0, 0.5), bc="bfs2d",
                              datum=False, mode="assemble", seed=3),
    # 3-D Boussinesq natural convection in a (perturbed) box
    "box3d_2x2x2_bouss": dict(mesh="hex27 2 2 2 1 1 1 0.1 5", phys="nst", rho=1.0,
                              visc=("newtonian", 0.71), bc="cube_heated", datum=True,
                              mode="assemble", seed=4, ra_pr=71000.0),
    "box3d_2x1x3_carreau_t": dict(mesh="hex27 2 1 3 1 0.5 1.5 0.12 9", phys="nst", rho=3.0,
                                  visc=("carreau", 2.0, 0.1, 0.5, 2.0, 0.6),
                                  bc="cube_heated", datum=True, mode="assemble", seed=6,
                                  ra_pr=500.0),
    # energy + two dilute species with an Arrhenius source (configuration 5 physics)
    "box3d_2x2x2_species": dict(mesh="hex27 2 2 2 1 1 1 0.1 13", phys="nsty", rho=1.0,
                                visc=("newtonian", 0.71), bc="cube_species", datum=True,
                                mode="assemble", seed=7, ra_pr=710.0, nspec=2,
                                diff=(0.05, 0.02), arrhenius=(3.0, 1.5), T_range=(1.0, 2.0)),
    # converged Newton solutions from a zero initial guess (T0: from that
    # temperature instead of zero)
    "box3d_2x2x2_species_solve": dict(mesh="hex27 2 2 2 1 1 1", phys="nsty", rho=1.0,
                                      visc=("newtonian", 0.71), bc="cube_species", datum=True,
                                      mode="solve", tol=1e-12, ra_pr=710.0, nspec=2,
                                      diff=(0.05, 0.02), arrhenius=(3.0, 1.5), T0=1.5),
    "cav2d_4x4_solve": dict(mesh="quad9 4 4 1 1", phys="ns", rho=100.0, visc=("newtonian", 1.0),
                            bc="cavity2d", datum=True, mode="solve", tol=1e-12),
    "cav2d_8x8_solve": dict(mesh="quad9 8 8 1 1", phys="ns", rho=100.0, visc=("newtonian", 1.0),
                            bc="cavity2d", datum=True, mode="solve", tol=1e-12),
    "bfs2d_6x2_carreau_solve": dict(mesh="quad9 6 2 3 1", phys="ns", rho=20.0,
                                    visc=("carreau", 1.0, 0.01, 1.0, 2.0, 0.5), bc="bfs2d",
                                    datum=False, mode="solve", tol=1e-12),
    "box3d_3x3x3_bouss_solve": dict(mesh="hex27 3 3 3 1 1 1", phys="nst", rho=1.0,
                                    visc=("newtonian", 0.71), bc="cube_heated", datum=True,
                                    mode="solve", tol=1e-12, ra_pr=7100.0),
    # the lid-driven cavity at its benchmark size (32 x 32 QUAD9, Re 100,
    # N = 11,522): compact records (every residual entry, a seeded sample of
    # Jacobian rows and a hash of the whole pattern; the converged solution)
    "cav2d_32x32": dict(mesh="quad9 32 32 1 1", phys="ns", rho=100.0, visc=("newtonian", 1.0),
                        bc="cavity2d", datum=True, mode="assemble", seed=8, compact=True),
    "cav2d_32x32_solve": dict(mesh="quad9 32 32 1 1", phys="ns", rho=100.0,
                              visc=("newtonian", 1.0), bc="cavity2d", datum=True, mode="solve",
                              tol=1e-10, compact=True),
    # transient: the first assembly of a time step (backward Euler, the
    # reference's first step) at a seeded state and time derivative, and a
    # fixed-step run from rest: three backward-Euler steps, then the deck's
    # Crank-Nicolson (theta 0.5) with its second-order predictor
    "cav2d_3x2_pert_transient": dict(mesh="quad9 3 2 1.5 1 0.15 7", phys="ns", rho=100.0,
                                     visc=("newtonian", 1.0), bc="cavity2d", datum=True,
                                     mode="assemble", seed=12,
                                     transient=dict(dt=0.05, steps=1, theta=0.5)),
    "box3d_2x2x2_bouss_transient": dict(mesh="hex27 2 2 2 1 1 1 0.1 5", phys="nst", rho=1.0,
                                        visc=("newtonian", 0.71), bc="cube_heated",
                                        datum=True, mode="assemble", seed=13, ra_pr=71000.0,
                                        transient=dict(dt=0.01, steps=1, theta=0.5)),
    "box3d_2x2x2_species_transient": dict(mesh="hex27 2 2 2 1 1 1 0.1 13", phys="nsty",
                                          rho=1.0, visc=("newtonian", 0.71),
                                          bc="cube_species", datum=True, mode="assemble",
                                          seed=14, ra_pr=710.0, nspec=2, diff=(0.05, 0.02),
                                          arrhenius=(3.0, 1.5), T_range=(1.0, 2.0),
                                          transient=dict(dt=0.02, steps=1, theta=0.5)),
    "cav2d_8x8_transient": dict(mesh="quad9 8 8 1 1", phys="ns", rho=100.0,
                                visc=("newtonian", 1.0), bc="cavity2d", datum=True,
                                mode="transient", tol=1e-12,
                                transient=dict(dt=0.02, steps=6, theta=0.5)),
    "box3d_2x2x2_bouss_transient_run": dict(mesh="hex27 2 2 2 1 1 1", phys="nst", rho=1.0,
                                            visc=("newtonian", 0.71), bc="cube_heated",
                                            datum=True, mode="transient", tol=1e-12,
                                            ra_pr=7100.0,
                                            transient=dict(dt=0.01, steps=5, theta=0.5)),
}

# integrated (weak) boundary conditions on side sets: a heat flux (QSIDE), a
# convective heat transfer (QCONV, h and T_inf) and an outflow pressure
# (FLOW_PRESSURE)
CASES.update({
    "channel2d_4x3_ibc": dict(mesh="quad9 4 3 2 1 0.12 17", phys="nst", rho=10.0,
                              visc=("newtonian", 1.0), bc="channel2d_t", datum=False,
                              mode="assemble", seed=16, ra_pr=0.0,
                              ibc=[("FLOW_PRESSURE", 2, (0.5,)), ("QCONV", 1, (2.0, 0.25)),
                                   ("QSIDE", 3, (0.7,))]),
    "box3d_2x2x2_ibc": dict(mesh="hex27 2 2 2 1 1 1 0.1 19", phys="nst", rho=1.0,
                            visc=("newtonian", 0.71), bc="box_open_top", datum=False,
                            mode="assemble", seed=17, ra_pr=710.0,
                            ibc=[("QCONV", 2, (2.0, 0.25)), ("QSIDE", 5, (0.7,)),
                                 ("FLOW_PRESSURE", 6, (0.3,))]),
    "channel2d_6x3_ibc_solve": dict(mesh="quad9 6 3 2 1", phys="nst", rho=10.0,
                                    visc=("newtonian", 1.0), bc="channel2d_t", datum=False,
                                    mode="solve", tol=1e-12, ra_pr=0.0,
                                    ibc=[("FLOW_PRESSURE", 2, (0.5,)),
                                         ("QCONV", 1, (2.0, 0.25)), ("QSIDE", 3, (0.7,))]),
})

# the Frank-Kamenetskii / Bratu problem: energy with the heat source
# c0 exp(c1 T) (a USER model, oracle/ref_shim/user_heat.c), T = 0 all round,
# the fluid at rest
CASES.update({
    "bratu2d_4x4_pert": dict(mesh="quad9 4 4 1 1 0.12 3", phys="nst", rho=1.0,
                             visc=("newtonian", 1.0), bc="bratu2d", datum=True,
                             mode="assemble", seed=15, ra_pr=0.0, heat=(5.0, 1.0)),
    "bratu2d_8x8_solve": dict(mesh="quad9 8 8 1 1", phys="nst", rho=1.0,
                              visc=("newtonian", 1.0), bc="bratu2d", datum=True, mode="solve",
                              tol=1e-12, ra_pr=0.0, heat=(5.0, 1.0)),
})

COMPACT_ROWS = 300  # Jacobian rows kept by a compact record

# Dirichlet sets: (variable, node set id, value), applied in this order
BCS = {
    "cavity2d": [("U", 1, 0.0), ("V", 1, 0.0), ("U", 2, 0.0), ("V", 2, 0.0), ("U", 4, 0.0),
                 ("V", 4, 0.0), ("U", 3, 1.0), ("V", 3, 0.0)],
    "bfs2d": [("U", 1, 0.0), ("V", 1, 0.0), ("U", 3, 0.0), ("V", 3, 0.0), ("U", 5, 0.0),
              ("V", 5, 0.0), ("U", 6, 1.0), ("V", 6, 0.0)],
    "cube_heated": [(c, s, 0.0) for s in (1, 2, 3, 4, 5, 6) for c in ("U", "V", "W")]
    + [("T", 1, 1.0), ("T", 2, 0.0)],
    # channel: walls y = 0 and y = Ly, plug inflow u = 1 with T = 1 at x = 0,
    # the outflow x = Lx left to an integrated condition
    "channel2d_t": [("U", 1, 0.0), ("V", 1, 0.0), ("U", 3, 0.0), ("V", 3, 0.0),
                    ("U", 4, 1.0), ("V", 4, 0.0), ("T", 4, 1.0)],
    # box: no-slip on the x and y faces, T = 1 at x = 0, the top z = Lz open
    "box_open_top": [(c, s, 0.0) for s in (1, 2, 3, 4, 5) for c in ("U", "V", "W")]
    + [("T", 1, 1.0)],
    "bratu2d": [(c, s, 0.0) for s in (1, 2, 4, 3) for c in ("U", "V")]
    + [("T", s, 0.0) for s in (1, 2, 3, 4)],
    # heated box with two species fed at x = 0: T in [1, 2] keeps exp(-E/T) finite
    "cube_species": [(c, s, 0.0) for s in (1, 2, 3, 4, 5, 6) for c in ("U", "V", "W")]
    + [("T", 1, 2.0), ("T", 2, 1.0), ("Y0", 1, 1.0), ("Y1", 1, 0.0)],
}


def time_cards(case):
    """Steady, or a fixed step (a negative delta_t keeps it constant,
    src/rf_solve.c:1153-1158) with the deck's time-step parameter theta."""
    tr = case.get("transient")
    if not tr:
        return ["Time integration = steady"]
    return ["Time integration = transient",
            "delta_t = %.17g" % (-tr["dt"]),
            "Maximum number of time steps = %d" % tr["steps"],
            "Maximum time = 1000.",
            "Minimum time step = 1.e-9",
            "Maximum time step = 10.",
            "Time step parameter = %.17g" % tr["theta"],
            "Time step error = 0.01 1 1 1 1 1 1 1",
            "Printing Frequency = 1"]


def deck_text(case):
    dim = 3 if case["mesh"].startswith("hex27") else 2
    newton = 1 if case["mode"] == "assemble" else 40
    lines = [
        "FEM File Specifications",
        "FEM file = mesh.exoII",
        "Output EXODUS II file = out.exoII",
        "GUESS file = guess.dat",
        "SOLN file = soln.dat",
        "Write intermediate results = no",
        "",
        "General Specifications",
        "Output Level = 0",
        "Debug = 0",
        "Initial Guess = zero",
        "",
        "Time Integration Specifications",
    ] + time_cards(case) + [
        "",
        "Solver Specifications",
        "Solution Algorithm = lu",
        "Matrix storage format = msr",
        "Number of Newton Iterations = %d" % newton,
        "Newton correction factor = 1",
        "Normalized Residual Tolerance = %g" % case.get("tol", 1e-10),
        "",
        "Boundary Condition Specifications",
        "Number of BC = %d" % len(BCS[case["bc"]]),
    ]
    for var, ns, val in BCS[case["bc"]]:
        if dim == 2 and var == "W":
            continue
        if var.startswith("Y"):      # species w: "BC = Y NS id w value"
            lines.append("BC = Y NS %d %d %.17g" % (ns, int(var[1:]), val))
        else:
            lines.append("BC = %s NS %d %.17g" % (var, ns, val))
    for name, ss, vals in case.get("ibc", []):   # integrated conditions on side sets
        lines.append("BC = %s SS %d %s" % (name, ss, " ".join("%.17g" % v for v in vals)))
    lines.append("END OF BC")
    if case["datum"]:
        lines += ["", "PRESSURE DATUM = 0 0."]
    lines += [
        "",
        "Problem Description",
        "Number of Materials = 1",
        "MAT = fluid 1",
        "Coordinate System = CARTESIAN",
        "Element Mapping = isoparametric",
        "Mesh Motion = ARBITRARY",
        "Number of bulk species = %d" % case.get("nspec", 0),
        "Number of EQ = -1",
    ]
    # the first term multiplier is the mass (time-derivative) term's
    mass = "1." if case.get("transient") else "0."
    for a in range(dim):
        lines.append("EQ = momentum%d Q2 U%d Q2 %s 1. 1. 1. 1. 0." % (a + 1, a + 1, mass))
    if case["phys"] in ("nst", "nsty"):
        lines.append("EQ = energy Q2 T Q2 %s 1. 1. 1. 1." % mass)
    if case["phys"] == "nsty":
        lines.append("EQ = species_bulk Q2 Y Q2 %s 1. 1. 1. 1." % mass)
    lines += ["EQ = continuity P1 P P1 1. 0.", "END OF EQ", "END OF MAT", "",
              "Post Processing Specifications", ""]
    # the BC count line must match what was written
    nbc = sum(1 for v, _, _ in BCS[case["bc"]] if not (dim == 2 and v == "W"))
    nbc += len(case.get("ibc", []))
    lines[lines.index("Number of BC = %d" % len(BCS[case["bc"]]))] = "Number of BC = %d" % nbc
    return "\n".join(lines)


def mat_text(case):
    visc = case["visc"]
    if visc[0] == "newtonian":
        vl = ["Liquid Constitutive Equation = NEWTONIAN", "Viscosity = CONSTANT %.17g" % visc[1]]
    else:
        _, mu0, muinf, lam, aexp, nexp = visc
        vl = ["Liquid Constitutive Equation = CARREAU", "Low Rate Viscosity = CONSTANT %.17g" % mu0,
              "Power Law Exponent = CONSTANT %.17g" % nexp,
              "High Rate Viscosity = CONSTANT %.17g" % muinf,
              "Time Constant = CONSTANT %.17g" % lam, "Aexp = CONSTANT %.17g" % aexp]
    if case["phys"] in ("nst", "nsty"):
        src = "Navier-Stokes Source = BOUSSINESQ 0. 0. %.17g" % (-case["ra_pr"])
    else:
        src = "Navier-Stokes Source = CONSTANT 0. 0. 0."
    return "\n".join([
        "---Physical Properties", "Density = CONSTANT %.17g" % case["rho"], "",
        "---Mechanical Properties and Constitutive Equations",
        "Solid Constitutive Equation = NONE", "Plasticity Equation = NONE",
        "Lame MU = CONSTANT 1.", "Lame LAMBDA = CONSTANT 1."] + vl + [
        "Polymer Constitutive Equation = NOPOLYMER", "",
        "---Thermal Properties", "Conductivity = CONSTANT 1.", "Heat Capacity = CONSTANT 1.",
        "Volume Expansion = CONSTANT 1.", "Reference Temperature = CONSTANT 0.5",
        "Liquidus Temperature = CONSTANT 0.", "Solidus Temperature = CONSTANT 0.", "",
        "---Electrical Properties", "Electrical Conductivity = CONSTANT 0.", "",
        "---Microstructure Properties", "Media Type = CONTINUOUS", "Porosity = CONSTANT 0.",
        "Permeability = CONSTANT 0.", "",
        ] + species_props(case) + [
        "---Source Terms", src, "Solid Body Source = CONSTANT 0. 0. 0.",
        "Mass Source = CONSTANT 0.", heat_source(case)] + species_sources(case) + [
        "Current Source = CONSTANT 0.", ""])


def heat_source(case):
    if "heat" in case:
        return "Heat Source = USER %.17g %.17g" % tuple(case["heat"])
    return "Heat Source = CONSTANT 0."


def species_props(case):
    ns = case.get("nspec", 0)
    if ns == 0:
        return ["---Species Properties", "Diffusion Constitutive Equation = NONE", ""]
    out = ["---Species Properties", "Diffusion Constitutive Equation = FICKIAN"]
    # the reader takes one group of cards per species, in species order
    for w in range(ns):
        out.append("Diffusivity = CONSTANT %d %.17g" % (w, case["diff"][w]))
        out += ["%s = CONSTANT %d 0." % (card, w)
                for card in ("Latent Heat Vaporization", "Latent Heat Fusion", "Vapor Pressure",
                             "Species Volume Expansion", "Reference Concentration")]
    return out + [""]


def species_sources(case):
    """Arrhenius: S_w = nu_w k0 exp(-E/T) Y_0 (USER model, oracle/ref_shim/user_species.c)."""
    ns = case.get("nspec", 0)
    out = []
    for w in range(ns):
        k0, E = case["arrhenius"]
        nu = -1.0 if w == 0 else 1.0
        out.append("Species Source = USER %d %.17g %.17g %.17g 0" % (w, k0, E, nu))
    return out


def temperature_unknowns(case):
    """Indices of the T unknowns (offset dim at every node, node-major DOF map)."""
    sys.path.insert(0, REPO)
    import oracle
    from tests import golden_cases as gc
    prob = gc.problem_from_case(case)
    fu = oracle.Oracle(prob).first_unknown(prob.mesh.num_nodes)
    return fu[:-1] + prob.dim


def run_case(name, case, outdir):
    with tempfile.TemporaryDirectory() as tmp:
        with open(os.path.join(tmp, "input"), "w") as f:
            f.write(deck_text(case))
        with open(os.path.join(tmp, "fluid.mat"), "w") as f:
            f.write(mat_text(case))
        env = dict(os.environ, GB_REF_MESH=case["mesh"], GB_REF_DUMP=os.path.join(tmp, "d"))
        rec = {"name": name, "case": json.dumps(case), "deck": deck_text(case),
               "mat": mat_text(case)}
        if case["mode"] == "assemble":
            # first pass: learn N from the dump of the zero state
            env1 = dict(env, GB_REF_EXIT="1")
            subprocess.run([GOMA, "-i", "input"], cwd=tmp, env=env1, check=True,
                           stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
            n = np.fromfile(os.path.join(tmp, "d.R")).size
            rng = np.random.default_rng(case["seed"])
            x = rng.uniform(-1.0, 1.0, n)
            if "T_range" in case:
                # temperatures inside a range (an Arrhenius rate needs T > 0)
                lo, hi = case["T_range"]
                x[temperature_unknowns(case)] = rng.uniform(lo, hi, len(temperature_unknowns(case)))
            x.astype("<f8").tofile(os.path.join(tmp, "xin.bin"))
            env2 = dict(env1, GB_REF_X_IN=os.path.join(tmp, "xin.bin"))
            if case.get("transient"):
                xd = rng.uniform(-1.0, 1.0, n)
                xd.astype("<f8").tofile(os.path.join(tmp, "xdin.bin"))
                env2["GB_REF_XDOT_IN"] = os.path.join(tmp, "xdin.bin")
            subprocess.run([GOMA, "-i", "input"], cwd=tmp, env=env2, check=True,
                           stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
            rec["x"] = np.fromfile(os.path.join(tmp, "d.x"))
            assert np.array_equal(rec["x"], x)
            if case.get("transient"):
                rec["xdot"] = np.fromfile(os.path.join(tmp, "d.xdot"))
                assert np.array_equal(rec["xdot"], xd)
                rec["delta_t_theta"] = np.fromfile(os.path.join(tmp, "d.dt"))
        else:
            if "T0" in case:
                # initial guess: Dirichlet values, T0 at the other temperatures
                # (zero everywhere else), as the package builds it
                sys.path.insert(0, REPO)
                import oracle
                from tests import golden_cases as gc
                o = oracle.Oracle(gc.problem_from_case(case))
                x0 = np.zeros(o.N)
                x0[temperature_unknowns(case)] = case["T0"]
                x0 = o.dirichlet_init(x0)
                x0.astype("<f8").tofile(os.path.join(tmp, "x0.bin"))
                env = dict(env, GB_REF_X_IN=os.path.join(tmp, "x0.bin"))
                rec["x0"] = x0
            p = subprocess.run([GOMA, "-i", "input"], cwd=tmp, env=env, check=True,
                               stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
            steady = case["mode"] == "solve"
            if steady and "converged SS!" not in p.stdout:
                raise RuntimeError("%s: reference Newton did not converge:\n%s" % (name, p.stdout[-3000:]))
            # the solution file: one block per printed step ("time = t"
            # first in a transient run)
            blocks, times = [[]], []
            with open(os.path.join(tmp, "soln.dat")) as f:
                for line in f:
                    parts = line.split()
                    if parts and parts[0] == "time":
                        if blocks[-1]:
                            blocks.append([])
                        times.append(float(parts[2]))
                    elif parts and parts[0][0] in "-0123456789":
                        blocks[-1].append(float(parts[0]))
            if steady:
                rec["x_converged"] = np.array(blocks[0])
            else:
                rec["x_steps"] = np.array(blocks)
                rec["times"] = np.array(times)
                if len(blocks) != case["transient"]["steps"]:
                    raise RuntimeError("%s: %d of %d time steps written:\n%s" % (
                        name, len(blocks), case["transient"]["steps"], p.stdout[-3000:]))
            rec["newton_log"] = "\n".join(l for l in p.stdout.splitlines() if "]" in l[:14])
            rec["x"] = np.fromfile(os.path.join(tmp, "d.x"))
        ija = np.fromfile(os.path.join(tmp, "d.ija"), dtype="<i4")
        a = np.fromfile(os.path.join(tmp, "d.a"))
        R = np.fromfile(os.path.join(tmp, "d.R"))
        if not case.get("compact"):
            rec["ija"], rec["a"], rec["R"] = ija, a, R
        else:
            rec.update(compact_record(case, ija, a, R))
    np.savez_compressed(os.path.join(outdir, name + ".npz"), **rec)
    return rec


def compact_record(case, ija, a, R):
    """What a large case keeps: N, the msr length, a SHA-256 of the whole
    pattern, and -- for assembly cases -- every residual entry and a seeded
    sample of Jacobian rows (diagonal first, then the off-diagonal columns
    in MSR order)."""
    import hashlib
    n = R.size
    out = {"N": np.int64(n), "msr_len": np.int64(ija[n]),
           "ija_sha256": hashlib.sha256(ija.astype("<i4").tobytes()).hexdigest()}
    if case["mode"] != "assemble":
        return out
    rng = np.random.default_rng(case["seed"] + 1000)
    rows = np.unique(np.concatenate([np.arange(8), np.arange(n - 8, n),
                                     rng.choice(n, COMPACT_ROWS, replace=False)]))
    ptr, cols, vals = [0], [], []
    for i in rows:
        cols += [i] + list(ija[ija[i]:ija[i + 1]])
        vals += [a[i]] + list(a[ija[i]:ija[i + 1]])
        ptr.append(len(cols))
    out.update(R=R, rows=rows.astype(np.int32), row_ptr=np.array(ptr, np.int32),
               row_cols=np.array(cols, np.int32), row_vals=np.array(vals))
    return out


NUMJAC = os.path.join(HERE, "numjac_reference.json")


def run_numjac(name, case):
    """The reference's own analytic-Jacobian checker (numerical_jacobian,
    src/mm_numjac.c:716, its default bracketed form) run by the reference on
    an assembly case at the case's seeded state: the deck's Debug = -2 makes
    solve_nonlinear_problem call it on its first step (rows scaled by their
    row sums; src/mm_sol_nonlinear.c:1194-1216) and exit.  Returns the
    entries it flags: the lines it prints for a perturbed residual outside
    the band the analytic Jacobians allow, and its dependency warnings."""
    g = np.load(os.path.join(HERE, name + ".npz"))
    with tempfile.TemporaryDirectory() as tmp:
        with open(os.path.join(tmp, "input"), "w") as f:
            f.write(deck_text(case).replace("Debug = 0", "Debug = -2"))
        with open(os.path.join(tmp, "fluid.mat"), "w") as f:
            f.write(mat_text(case))
        g["x"].astype("<f8").tofile(os.path.join(tmp, "x.bin"))
        env = dict(os.environ, GB_REF_MESH=case["mesh"], GB_REF_X_IN=os.path.join(tmp, "x.bin"))
        p = subprocess.run([GOMA, "-i", "input"], cwd=tmp, env=env, check=True,
                           capture_output=True, text=True)
    if "numerical Jacobian done" not in p.stdout:
        raise RuntimeError("%s: the reference's checker did not finish:\n%s" % (name, p.stdout[-2000:]))
    flagged = [l.strip() for l in p.stderr.splitlines()
               if "conf=" in l or "Potential dependency error" in l]
    return {"columns": int(g["x"].size), "debug_flag": -2, "flagged": flagged}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("GOMA_REFERENCE", "/root/reference"),
                    help="reference source root (default: $GOMA_REFERENCE)")
    ap.add_argument("--numjac", action="store_true",
                    help="run the reference's Jacobian checker on the (non-compact) assembly "
                         "cases into numjac_reference.json instead")
    ap.add_argument("cases", nargs="*")
    args = ap.parse_args()
    if not os.path.exists(GOMA):
        subprocess.run([os.path.join(REPO, "oracle", "build_ref.sh"), args.ref], check=True)
    if args.numjac:
        names = args.cases or [n for n, c in CASES.items()
                               if c["mode"] == "assemble" and not c.get("compact")]
        out = {}
        if os.path.exists(NUMJAC):
            with open(NUMJAC) as f:
                out = json.load(f)
        for name in names:
            out[name] = run_numjac(name, CASES[name])
            print("%-28s columns=%5d flagged=%d" % (name, out[name]["columns"],
                                                     len(out[name]["flagged"])))
        with open(NUMJAC, "w") as f:
            json.dump(out, f, indent=1, sort_keys=True)
        return 0
    names = args.cases or list(CASES)
    for name in names:
        rec = run_case(name, CASES[name], HERE)
        if "ija" in rec:
            n = rec["R"].size
            ml = rec["ija"][n]
        else:
            n, ml = int(rec["N"]), int(rec["msr_len"])
        print("%-28s N=%6d msr_len=%8d %s" % (name, n, ml, CASES[name]["mode"]))


if __name__ == "__main__":
    sys.exit(main())
