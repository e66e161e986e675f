"""Benchmark of the Q2/P1 Newton hot path on one GB300.

Workload: 3-D Boussinesq natural convection in a unit cube, 32^3 HEX27
elements, Q2 velocity + temperature / P1 pressure (1,229,572 unknowns,
300,429,328 CSR nonzeros), the configuration the headline metric is quoted
on.  A step is one full residual + analytic-Jacobian assembly
(matrix_fill_full): zeroing, the element kernels and the coloured CSR
scatter, at a seeded synthetic state.

  value  elements/s with x, R and the matrix resident in HBM
  e2e    elements/s through the C ABI with host buffers: x copied in, R and
         the Jacobian (reference MSR layout) copied out, every step
  roofline  the element kernel: the FP64 operations its algorithm performs
         per launch (element_flops) / measured kernel time, against this
         GPU's FP64 throughput measured in-process (scalar FMA and mma.sync
         f64 run at the same rate); the dense-equivalent rate and the HBM
         view of the same launch alongside
  cpu_baseline  the CPU oracle (the golden-pinned restatement of the
         reference's matrix_fill_full) assembling the same 32^3 workload on
         all host threads

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Q2/P1 elem/s (R+J); time-to-solve @1e-8, plain vs learned+FP32 GMRES, 1 GB300"
UNIT = "elements/s"
NEL = 32
RA, PR = 1e5, 0.71


def workload_config(nel):
    return {"workload": "3-D Boussinesq cube %d^3 HEX27 Q2/P1 NS+energy, Ra=1e5 Pr=0.71" % nel,
            "elements": nel ** 3, "element": "HEX27", "fields": "u,v,w,T (Q2), P (P1)",
            "state": "seeded uniform(-1,1) unknowns", "assembly": "R + analytic J, FP64",
            "l2": "inputs larger than L2 (CSR values 2.4 GB)"}


def read_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "source": "fallback"}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    def __init__(self):
        self.rows = []
        self.proc = None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0],
                 "--query-gpu=" + q, "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            p = [s.strip() for s in line.split(",")]
            if len(p) == 7:
                self.rows.append(p)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait(timeout=5)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4)
                          if r[3 + i].lower().startswith("active")})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.rows)}


class CpuAssembly:
    """The reference's CPU assembly of the whole nel^3 workload, timed: the
    CPU oracle (the golden-pinned restatement of the reference's
    matrix_fill_full, not Goma itself) over `threads` host threads, each
    step the caller's zeroing of R and the 2.5 GB of MSR values and all
    nel^3 elements, colour by colour, into one shared MSR array
    (oracle.ParallelFill)."""

    def __init__(self, nel, threads):
        import oracle
        from goma_gb300 import problem as pb
        t = time.perf_counter()
        self.nel = nel
        self.o = oracle.Oracle(pb.boussinesq_cube_3d(nel, RA, PR))
        self.fill = oracle.ParallelFill(self.o, threads)
        self.x = self.o.dirichlet_init(np.random.default_rng(11).uniform(-1.0, 1.0, self.o.N))
        self.setup_s = time.perf_counter() - t

    def step(self):
        t = time.perf_counter()
        if self.fill(self.x) != 0:
            raise RuntimeError("CPU assembly: non-positive Jacobian determinant")
        return time.perf_counter() - t

    def describe(self, steps, dt):
        return ("CPU oracle matrix_fill_full (golden-pinned restatement of the reference's, "
                "not Goma itself) over the whole %d^3 HEX27 Boussinesq workload (%d elements, "
                "zeroing of R and the MSR values included), %d colours, element chunks over %d "
                "host threads into one MSR array; %d step(s), %.2f s each"
                % (self.nel, self.nel ** 3, self.fill.num_colors, self.fill.threads, steps, dt))

    def close(self):
        self.fill.close()


def cpu_baseline(nel=NEL, threads=None, steps=1):
    """The reference's CPU assembly of the same workload on the host cores:
    one untimed pass (pages the arrays in), then `steps` timed passes."""
    threads = threads or os.cpu_count() or 1
    ca = CpuAssembly(nel, threads)
    ca.step()
    dts = [ca.step() for _ in range(steps)]
    dt = float(np.median(dts))
    out = {"value": nel ** 3 / dt, "unit": UNIT, "cores": threads, "kind": "port",
           "sample": ca.describe(steps, dt), "setup_s": ca.setup_s}
    ca.close()
    return out


def time_to_solve(nel, ra0=1e4, ra1=1e5, nsteps=6, tol=1e-10, ilu_ordering=-1, krylov=300,
                  forcing=1, reference_solver=True, modes=None, budget_s=None,
                  factorization_reuse=0, max_linear_its=4000, inner_tol=1e-3):
    """Wall-clock time to the converged Boussinesq cube at Ra = ra1, by Ra
    continuation from rest at Ra = ra0 in nsteps log-uniform steps: plain
    FP64 Newton (ILU(0)-GMRES in FP64, zeroth-order predictor, the
    reference's ALC_ZEROTH) against the learned predictor (secant fallback)
    with FP64 GMRES and with FP32 GMRES: the _fp32 runs are FP64 flexible
    GMRES with the ILU(0) factorised and swept in FP32, the _fp32r runs FP32
    GMRES inside FP64 iterative refinement; the secant_fp32 run is the
    learned_fp32 run without the network (the plain secant guess), so the
    two isolate what the network gains.  All use the same
    linear-solver settings: ILU(0), GMRES(krylov), Eisenstat-Walker forcing
    (the converged solution does not depend on them).  ilu_ordering -1
    chooses the node order by size: the multicoloured one up to 12^3 (few
    dependency levels, cheap iterations), the reference's above (its
    iteration count grows far more slowly: 801 against 4,198 Krylov
    iterations for one 16^3 solve, 2,441 against 24,600 at 24^3).  With reference_solver the plain FP64
    run is repeated with the reference's settings (ILU(0) in its node
    order, GMRES(30), every linear solve to 1e-8).  `modes` selects runs;
    `budget_s` ends each run's sweep after that many seconds (reported as
    steps done).  factorization_reuse (GB_FACTOR_*) applies to every run
    but the one with the reference's settings; inner_tol is the FP32 runs'
    tightest inner tolerance.  Returns a dict with the times, Newton/Krylov counts,
    per-phase splits and the relative difference of the converged
    solutions."""
    if ilu_ordering < 0:
        ilu_ordering = 1 if nel <= 12 else 0
    import torch
    from goma_gb300 import problem as pb
    from goma_gb300.continuation import continuation
    from goma_gb300.newton import GomaNewton

    def set_ra(gn, ra):
        m = gn.problem.material
        m.momentum_source = (0.0, 0.0, -ra * PR)
        gn.set_material(m)

    out = {"workload": "%d^3 HEX27 Boussinesq cube, Ra %g -> %g in %d log-uniform continuation "
                       "steps from rest, Pr=%g, scaled |R| < %g" % (nel, ra0, ra1, nsteps, PR, tol),
           "linear_solver": "ILU(0) in the %s node order, GMRES(%d), %s, factors %s; the _fp32 "
                            "runs: FP64 flexible GMRES with the ILU(0) factorised and swept in "
                            "FP32" % (
               "reference's" if ilu_ordering == 0 else "multicoloured", krylov,
               "Eisenstat-Walker forcing (1e-8 .. 1e-2)" if forcing else "linear tol 1e-8",
               ["at every Newton step", "once per Newton solve", "reused across solves"][
                   factorization_reuse])}
    # first-use costs of the process (CUDA module loading of the network and
    # copy kernels) are paid once here, outside both timed runs
    from goma_gb300.mlp import GpuMLP
    warm = GpuMLP(4, 32, 2, 1, seed=1)
    xw = torch.zeros((64, 4), device="cuda")
    tw = torch.zeros((64, 1), device="cuda")
    warm.train(xw, tw, torch.ones_like(tw), steps=2, batch=32)
    warm.forward(xw).cpu().numpy()
    torch.cuda.synchronize()
    del warm, xw, tw
    sols = {}
    modes = list(modes) if modes else ["plain_fp64", "secant_fp32", "learned_fp32"] + (
        ["plain_fp64_reference_solver"] if reference_solver else [])
    for mode in modes:
        prob = pb.boussinesq_cube_3d(nel, ra0, PR)
        gn = GomaNewton(prob)
        refs = mode == "plain_fp64_reference_solver"
        gn.set_ilu_ordering(0 if refs else ilu_ordering)
        opts = dict(residual_tol=tol, linear_tol=1e-8, max_newton=30,
                    max_linear_its=max_linear_its,
                    fp32_preconditioner=mode.endswith("_fp32"),
                    fp32_inner=mode.endswith("_fp32r"), inner_tol=inner_tol,
                    krylov_dim=30 if refs else krylov, forcing=0 if refs else forcing,
                    forcing_max=1e-2, factorization_reuse=0 if refs else factorization_reuse)
        torch.cuda.synchronize()
        t = time.perf_counter()
        recs, x = continuation(gn, ra0, ra1, nsteps,
                               predictor={"plain": "zeroth", "secant": "secant",
                                          "learned": "learned"}[mode.split("_")[0]],
                               set_param=set_ra, newton_opts=opts, spacing="log",
                               learned_opts=dict(steps=300, batch=4096, lr=2e-3,
                                                 warm_steps=75),
                               time_budget_s=budget_s)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t
        sols[mode] = x
        ms = {k: sum(r["newton_ms"][k] for r in recs) for k in recs[0]["newton_ms"]}
        out[mode] = {"seconds": dt, "steps_done": len(recs) - 1, "last_ra": recs[-1]["lam"],
                     "newton_its": sum(r["newton_its"] for r in recs),
                     "linear_its": sum(r.get("linear_its", 0) for r in recs),
                     "factorizations": sum(r.get("factorizations", 0) for r in recs),
                     "guesses": [r["guess"] for r in recs[1:]],
                     "newton_seconds": {k.replace("_ms", ""): v * 1e-3 for k, v in ms.items()},
                     "predictor_seconds": sum(r.get("predictor_s", 0.0) for r in recs),
                     "candidate_seconds": sum(r.get("candidates_s", 0.0) for r in recs),
                     "candidate_residual_seconds": sum(r.get("residuals_s", 0.0) for r in recs),
                     "training_seconds": sum(r.get("train_s", 0.0) for r in recs)}
        out[mode]["newton_steps_per_s"] = out[mode]["newton_its"] / dt
        del gn
    a = sols.get("plain_fp64")
    complete = {m for m in sols if out[m]["steps_done"] == nsteps}
    for m in sols:
        if m != "plain_fp64" and a is not None and {m, "plain_fp64"} <= complete:
            out["solution_rel_diff_" + m] = float(np.abs(a - sols[m]).max() / np.abs(a).max())
            out["speedup_" + m] = out["plain_fp64"]["seconds"] / out[m]["seconds"]
    # the network's own gain: the same FP32-inner solve with the plain secant
    # guess in its place
    if {"secant_fp32", "learned_fp32"} <= complete:
        out["learned_over_secant_seconds"] = (out["learned_fp32"]["seconds"] /
                                              out["secant_fp32"]["seconds"])
    if "speedup_learned_fp32" in out:
        out["speedup"] = out["speedup_learned_fp32"]
        out["solution_rel_diff"] = out["solution_rel_diff_learned_fp32"]
    return out


def element_flops(path):
    """FP64 operations (FMA = 2) per 32^3-workload element (HEX27, NS + energy,
    Jacobian) of the element kernel of `path`, counted from its algorithm.

    Path 4 (sum factorisation, the automatic path): isoparametric passes
    7 fields x (2 + 3 + 4) x 27 outputs x 5; per-point set-up ~263 x 27;
    gradient tables 729 x 18; sum-factorisation stages 16 x (81 + 243) x 5;
    residual rows 108 x 27 x 8; J_mP 324 x 27 x 2; upper triangle of the
    81 x 81 gradient product 3,321 x 27 x 2; node pairs 729 x 113.
    Paths 1-3 do the dense quadrature-point contractions: 2 Q n_loc^2 (d+1)."""
    if path in (0, 4):
        iso = 7 * (2 + 3 + 4) * 27 * 5
        qp = 263 * 27
        tables = 729 * 18
        stages = 16 * (81 + 243) * 5
        resid = 108 * 27 * 8
        jmp = 324 * 27 * 2
        h = 3321 * (27 * 2 + 2)
        pairs = 729 * 113
        return float(iso + qp + tables + stages + resid + jmp + h + pairs)
    nloc = 4 * 27 + 4
    return 2.0 * 27 * nloc * nloc * 4


def reacting_channel_assembly(nx, ny, nz, steps=3, warmup=2):
    """Device-resident assembly throughput of the reacting channel (HEX27 Q2/P1
    Navier-Stokes + energy + 2 Arrhenius species, 7.0 M unknowns and 2.6e9
    CSR nonzeros at 64 x 64 x 32), timed with CUDA events on the library's
    stream, into the library's own device buffers (no second copy of the
    values).  The reference's 32-bit MSR indexing cannot hold this size."""
    import time as _time

    import torch
    from goma_gb300 import problem as pb
    from goma_gb300.newton import GomaNewton
    t0 = _time.perf_counter()
    prob = pb.reacting_channel_3d(nx, ny, nz, seed=0)
    gn = GomaNewton(prob)
    setup_s = _time.perf_counter() - t0
    rng = np.random.default_rng(5)
    x = gn.dirichlet_init(rng.uniform(0.5, 1.5, gn.N))
    dx = torch.tensor(x, dtype=torch.float64, device="cuda")
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream

    def step():
        gn.matrix_fill_full_device(dx.data_ptr(), gn.d_R, gn.d_vals, sp)

    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    gn.status()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    gn.status()
    ms = e0.elapsed_time(e1) / steps
    ne = prob.mesh.num_elems
    out = {"workload": "reacting channel %dx%dx%d HEX27 Q2/P1 NS + energy + 2 Arrhenius "
                       "species (D=1e-3, k0=%.3f seeded), seeded state" %
                       (nx, ny, nz, prob.material.species_source[0][1][0]),
           "elements": ne, "unknowns": gn.N, "csr_nnz": gn.nnz,
           "ms_per_assembly": ms, "elements_per_s": ne / (ms * 1e-3),
           "layout_and_upload_s": setup_s, "colors": gn.num_colors,
           "note": "device-resident R + analytic J; flow rows by the sum-factorised kernel, "
                   "species rows by the species kernel"}
    del dx
    gn.close()
    torch.cuda.empty_cache()
    return out


def reacting_channel_solve(nx=64, ny=64, nz=32, tol=1e-8, max_newton=15, max_linear_its=2000,
                           krylov=150):
    """The reacting channel (HEX27 Q2/P1 Navier-Stokes + energy + 2 Arrhenius
    species, 7.0 M unknowns at 64 x 64 x 32) solved by Newton from the inflow
    state (u = 1, T = 1.5, Y_0 = 1, Y_1 = 0 inside, the Dirichlet values on
    the boundary) to the scaled residual `tol`, with FP64 flexible GMRES
    whose ILU(0) preconditioner is factorised and swept in FP32, and
    Eisenstat-Walker forcing: time, Newton and
    Krylov counts and the per-phase split.  The reference's 32-bit MSR cannot
    hold this problem."""
    import time as _time

    import torch
    from goma_gb300 import problem as pb
    from goma_gb300.newton import GomaNewton
    t0 = _time.perf_counter()
    prob = pb.reacting_channel_3d(nx, ny, nz, seed=0)
    gn = GomaNewton(prob)
    gn.set_ilu_ordering(0)
    setup_s = _time.perf_counter() - t0
    fu = np.empty(prob.mesh.num_nodes + 1, np.int32)
    from goma_gb300 import _lib
    _lib.check(gn._L.gb_first_unknown(gn.h, fu.ctypes.data_as(ctypes.POINTER(ctypes.c_int))))
    x = np.zeros(gn.N)
    x[fu[:-1] + 0] = 1.0          # u
    x[fu[:-1] + 3] = 1.5          # T
    x[fu[:-1] + 4] = 1.0          # Y_0
    x = gn.dirichlet_init(x)
    torch.cuda.synchronize()
    t1 = _time.perf_counter()
    x, conv, st = gn.solve_nonlinear_problem(
        x, residual_tol=tol, linear_tol=1e-8, max_newton=max_newton,
        max_linear_its=max_linear_its, krylov_dim=krylov, fp32_preconditioner=True,
        forcing=1, forcing_max=1e-2)
    torch.cuda.synchronize()
    dt = _time.perf_counter() - t1
    out = {"workload": "reacting channel %dx%dx%d HEX27 Q2/P1 NS + energy + 2 Arrhenius species, "
                       "Newton from the inflow state to scaled |R| < %g, FP64 flexible "
                       "GMRES(%d) with FP32 ILU(0), forcing rule" % (nx, ny, nz, tol, krylov),
           "unknowns": gn.N, "csr_nnz": gn.nnz, "converged": conv, "seconds": dt,
           "layout_and_upload_s": setup_s, "newton_its": st["newton_its"],
           "linear_its": st["linear_its"], "residual_l2": st["residual_l2"],
           "newton_seconds": {k.replace("_ms", ""): st[k] * 1e-3
                              for k in ("assemble_ms", "scale_ms", "factor_ms", "solve_ms",
                                        "total_ms")}}
    print("reacting_solve:", {k: out[k] for k in ("converged", "seconds", "newton_its",
                                                  "linear_its")}, file=sys.stderr, flush=True)
    gn.close()
    torch.cuda.empty_cache()
    return out


def batch_sweep_assembly(num=512, seed=0, steps=3, warmup=2):
    """Assembly throughput of the 512-problem sweep held as one union: one
    launch per colour over every problem's elements, per-element Reynolds
    numbers, device-resident R + analytic J."""
    import time as _time

    import torch
    from goma_gb300 import problem as pb
    from goma_gb300.newton import GomaNewton
    t0 = _time.perf_counter()
    b = pb.batch_sweep_2d(num, seed=seed)
    gn = GomaNewton(b.problem)
    gn.set_element_density(b.elem_re)
    setup_s = _time.perf_counter() - t0
    x = gn.dirichlet_init(np.random.default_rng(3).uniform(-1, 1, gn.N))
    dx = torch.tensor(x, dtype=torch.float64, device="cuda")
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream
    for _ in range(warmup):
        gn.matrix_fill_full_device(dx.data_ptr(), gn.d_R, gn.d_vals, sp)
    torch.cuda.synchronize()
    gn.status()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        gn.matrix_fill_full_device(dx.data_ptr(), gn.d_R, gn.d_vals, sp)
    e1.record(stream)
    torch.cuda.synchronize()
    gn.status()
    ms = e0.elapsed_time(e1) / steps
    ne = b.problem.mesh.num_elems
    out = {"workload": "%d unit-square QUAD9 Q2/P1 problems (cavity / channel), n x n with n "
                       "uniform in [16, 64], Re log-uniform in [10, 1000], seed %d, one context"
                       % (num, seed),
           "elements": ne, "unknowns": gn.N, "csr_nnz": gn.nnz, "colors": gn.num_colors,
           "ms_per_assembly": ms, "elements_per_s": ne / (ms * 1e-3),
           "launches_per_assembly": gn.num_colors, "layout_and_upload_s": setup_s}
    del dx
    gn.close()
    torch.cuda.empty_cache()
    return out


def batch_sweep_solve(num=64, seed=0, stages=2, tol=1e-10, fp32_inner=False, check=2,
                      ilu_ordering=0, budget_s=240.0, nmin=16, nmax=32, re_max=100.0,
                      max_ratio=None, max_linear_its=600, fp32_preconditioner=False):
    """The 512-problem sweep: unit-square QUAD9 Q2/P1 cavities and channels,
    meshes n x n with n uniform in [16, 64], Re log-uniform in [10, 1000]
    (seeded), all held in one context as a disjoint union with per-element
    Reynolds numbers, so one assembly launch per colour and one Krylov solve
    serve every problem.  Newton from rest to the scaled residual `tol`,
    through `stages` geometric Reynolds ramps (Re_p 10^(k/stages) ... up to
    each problem's own Re).  With max_ratio the number of stages is chosen
    so that no problem's Re grows by more than that factor from one stage to
    the next (Newton from the previous stage's solution converges in 4-5
    steps for ratios up to ~1.7 on cavities up to Re 1000; a 10x step from
    Re 100 diverges).  The Krylov solve is the batched GMRES (one
    Arnoldi process per problem).  `check` of the smallest members are solved
    again, on their own, by the CPU oracle, and compared.  Stages stop once
    `budget_s` seconds have passed (reported as not converged)."""
    import time as _time

    import torch
    from goma_gb300 import problem as pb
    from goma_gb300.newton import GomaNewton
    t0 = _time.perf_counter()
    b = pb.batch_sweep_2d(num, seed=seed, nmin=nmin, nmax=nmax, re_max=re_max)
    if max_ratio is not None:
        stages = max(1, int(np.ceil(np.log(b.elem_re.max() / 10.0) / np.log(max_ratio))))
    gn = GomaNewton(b.problem)
    gn.set_ilu_ordering(ilu_ordering)
    setup_s = _time.perf_counter() - t0
    re = b.elem_re
    x = None
    recs = []
    torch.cuda.synchronize()
    t1 = _time.perf_counter()
    for k in range(stages + 1):
        rho = np.minimum(re, 10.0 * (re / 10.0) ** (k / stages)) if stages else re
        gn.set_element_density(rho)
        if _time.perf_counter() - t1 > budget_s:
            recs.append({"stage": k, "converged": False, "skipped": "time budget"})
            break
        ts = _time.perf_counter()
        x, conv, st = gn.solve_nonlinear_problem(
            x, residual_tol=tol, linear_tol=1e-8, max_newton=15, max_linear_its=max_linear_its,
            fp32_inner=fp32_inner, fp32_preconditioner=fp32_preconditioner, inner_tol=1e-3,
            forcing=1, forcing_max=1e-2)
        print("batch stage %d: converged %s, %d Newton, %d Krylov, %.1f s, |R| %s" % (
            k, conv, st["newton_its"], st["linear_its"], _time.perf_counter() - ts,
            st["residual_l2"][-1] if st["residual_l2"] else None), file=sys.stderr, flush=True)
        recs.append({"stage": k, "converged": conv, "newton_its": st["newton_its"],
                     "linear_its": st["linear_its"],
                     "newton_seconds": {kk.replace("_ms", ""): st[kk] * 1e-3
                                        for kk in ("assemble_ms", "factor_ms", "solve_ms",
                                                   "total_ms")}})
        if not conv:
            break
    torch.cuda.synchronize()
    solve_s = _time.perf_counter() - t1
    nelem = b.problem.mesh.num_elems
    out = {"workload": "%d unit-square QUAD9 Q2/P1 problems (cavity / channel), n x n with n "
                       "uniform in [%d, %d], Re log-uniform in [10, %g], seed %d, one context"
                       % (num, nmin, nmax, re_max, seed),
           "elements": nelem, "unknowns": gn.N, "csr_nnz": gn.nnz,
           "seconds_to_solve_all": solve_s, "layout_and_upload_s": setup_s,
           "converged": all(r["converged"] for r in recs), "stages": recs,
           "fp32_inner": fp32_inner, "fp32_preconditioner": fp32_preconditioner,
           "ilu_order": "multicoloured" if ilu_ordering == 1 else "the reference's"}
    if check and out["converged"]:
        import oracle
        ctypes_fu = np.empty(b.problem.mesh.num_nodes + 1, np.int32)
        from goma_gb300 import _lib
        _lib.check(gn._L.gb_first_unknown(gn.h, ctypes_fu.ctypes.data_as(
            ctypes.POINTER(ctypes.c_int))))
        diffs = []
        for p in sorted(range(num), key=lambda q: b.members[q].n)[:check]:
            mb = b.members[p]
            lo, hi = ctypes_fu[mb.nodes[0]], ctypes_fu[mb.nodes[1]]
            o = oracle.Oracle(pb.batch_member_problem(b, p))
            xo = None
            for k in range(stages + 1):   # the oracle follows the same Re ramp
                rr = min(mb.re, 10.0 * (mb.re / 10.0) ** (k / stages)) if stages else mb.re
                pp = pb.batch_member_problem(b, p)
                pp.material.density = rr
                o = oracle.Oracle(pp)
                xo, _, _ = o.newton(o.dirichlet_init(np.zeros(o.N) if xo is None else xo))
            diffs.append({"member": p, "kind": mb.kind, "n": mb.n, "re": mb.re,
                          "rel_diff": float(np.abs(x[lo:hi] - xo).max() / np.abs(xo).max())})
        out["oracle_check"] = diffs
    gn.close()
    torch.cuda.empty_cache()
    return out


def cpu_time_to_solve(nel=8, ra0=1e4, ra1=1e5, nsteps=6, tol=1e-10, krylov=30, linear_tol=1e-8):
    """The time-to-solve continuation of `time_to_solve` (Ra ra0 -> ra1 in
    nsteps log-uniform steps from rest, zeroth-order predictor, scaled
    |R| < tol) on one host core: the CPU oracle's assembly (restatement of
    the reference's matrix_fill), row-sum scaling and Newton loop with its
    ILU(0)-GMRES(krylov) restatement at the reference's solver settings
    (natural node order, every linear solve to linear_tol).  The reference's
    own Krylov solver (AztecOO) is third-party and not built here, so this
    is labelled "not AztecOO"; it pairs with the GPU's
    plain_fp64_reference_solver run of the same sweep."""
    import dataclasses

    import oracle
    from goma_gb300 import problem as pb
    prob = pb.boussinesq_cube_3d(nel, ra0, PR)
    x = None
    recs = []
    t0 = time.perf_counter()
    for k, ra in enumerate(np.geomspace(ra0, ra1, nsteps + 1)):
        mat = dataclasses.replace(prob.material, momentum_source=(0.0, 0.0, -ra * PR))
        o = oracle.Oracle(dataclasses.replace(prob, material=mat))
        if x is None:
            x = o.dirichlet_init(np.zeros(o.N))
        ts = time.perf_counter()
        x, it, lin, _ = o.newton_gmres(x, 40, tol, linear_tol=linear_tol, krylov=krylov,
                                       max_linear_its=4000)
        recs.append({"ra": float(ra), "newton_its": int(it), "linear_its": int(lin),
                     "seconds": time.perf_counter() - ts})
        if it < 0:
            break
    out = {"workload": "%d^3 HEX27 Boussinesq cube, Ra %g -> %g in %d log-uniform continuation "
                       "steps from rest, Pr=%g, scaled |R| < %g" % (nel, ra0, ra1, nsteps, PR, tol),
           "solver": "CPU oracle: ILU(0) (natural order) + GMRES(%d) restatement, not AztecOO, "
                     "every linear solve to %g, 1 thread" % (krylov, linear_tol),
           "seconds": time.perf_counter() - t0, "cores": 1,
           "converged": all(r["newton_its"] >= 0 for r in recs) and len(recs) == nsteps + 1,
           "newton_its": sum(max(r["newton_its"], 0) for r in recs),
           "linear_its": sum(r["linear_its"] for r in recs), "steps": recs}
    out["newton_steps_per_s"] = out["newton_its"] / out["seconds"]
    return out


def factorization_reuse_solves(nel=16, ra=1e4, tol=1e-10, fp32=False):
    """One Newton solve of the Boussinesq cube from rest (Ra `ra`, GMRES(60),
    forcing rule, the reference's node order) with each factorisation reuse
    mode (0 every Newton step, 1 once per solve, 2 across solves, after a
    first solve): wall time, Newton and Krylov counts and factorisations."""
    import time as _time

    import torch
    from goma_gb300 import problem as pb
    from goma_gb300.newton import GomaNewton
    rows = []
    gn = GomaNewton(pb.boussinesq_cube_3d(nel, ra, PR))
    gn.set_ilu_ordering(0)
    for reuse in (0, 1, 2):
        torch.cuda.synchronize()
        t = _time.perf_counter()
        x, conv, st = gn.solve_nonlinear_problem(
            residual_tol=tol, linear_tol=1e-8, max_newton=30, max_linear_its=4000,
            krylov_dim=60, forcing=1, forcing_max=1e-2, fp32_inner=fp32,
            factorization_reuse=reuse)
        torch.cuda.synchronize()
        rows.append({"factorization_reuse": reuse, "converged": conv,
                     "seconds": _time.perf_counter() - t, "newton_its": st["newton_its"],
                     "linear_its": st["linear_its"], "factorizations": st["factorizations"],
                     "factor_seconds": st["factor_ms"] * 1e-3,
                     "solve_seconds": st["solve_ms"] * 1e-3})
        print("reuse:", rows[-1], file=sys.stderr, flush=True)
    gn.close()
    return {"workload": "%d^3 Boussinesq cube Newton solve from rest, Ra %g, GMRES(60), "
                        "forcing rule, %s" % (nel, ra, "FP32 inner" if fp32 else "FP64"),
            "runs": rows}


def ilu_orders(sizes=(8, 16, 24), ra=1e4, tol=1e-10):
    """One Newton solve of the Boussinesq cube from rest (Ra `ra`, scaled
    |R| < tol, GMRES(60), forcing rule) per cube size, ILU(0) node order
    (the reference's, multicoloured) and inner precision (FP64, FP32 up to
    16^3): wall time, Newton and Krylov counts and the Krylov phase's time per
    iteration (CUDA-event phase timers of the Newton driver)."""
    import time as _time

    import torch
    from goma_gb300 import problem as pb
    from goma_gb300.newton import GomaNewton
    rows = []
    for nel in sizes:
        prob = pb.boussinesq_cube_3d(nel, ra, PR)
        for ordering in (0, 1):
            for fp32 in ((False, True) if nel <= 16 else (False,)):
                gn = GomaNewton(prob)
                gn.set_ilu_ordering(ordering)
                torch.cuda.synchronize()
                t = _time.perf_counter()
                x, conv, st = gn.solve_nonlinear_problem(
                    residual_tol=tol, linear_tol=1e-8, max_newton=30, max_linear_its=4000,
                    krylov_dim=60, forcing=1, forcing_max=1e-2, fp32_inner=fp32)
                torch.cuda.synchronize()
                dt = _time.perf_counter() - t
                rows.append({"cube": nel, "ilu_order": "multicoloured" if ordering else
                             "the reference's", "fp32_inner": fp32, "converged": conv,
                             "seconds": dt, "newton_its": st["newton_its"],
                             "linear_its": st["linear_its"],
                             "ms_per_krylov_it": st["solve_ms"] / max(1, st["linear_its"]),
                             "factor_seconds": st["factor_ms"] * 1e-3})
                print("ilu_orders:", rows[-1], file=sys.stderr, flush=True)
                gn.close()
                del gn
                torch.cuda.empty_cache()
    return {"workload": "Boussinesq cube Newton solve from rest, Ra %g, scaled |R| < %g, "
                        "GMRES(60), Eisenstat-Walker forcing" % (ra, tol), "runs": rows}


def krylov_kernels(nel, iters=30, ra=1e4):
    """The linear-solver kernels on one Newton system of the nel^3
    Boussinesq cube (the state at rest, Ra `ra`), in the reference's node
    order with the sync-free sweeps: one Newton step each in FP64 and in
    FP32-inner mode, each a factorisation plus exactly `iters` GMRES(iters)
    iterations (tolerance out of reach), timed by the Newton driver's CUDA
    events.  Algorithmic bytes per launch, for the rooflines of the launch
    list: SpMV 12 nnz + 24 N (FP64) / 8 nnz + 12 N (FP32); one triangular
    sweep reads its factor's half of the values and column indices, the
    right-hand side and writes the solution (about (8 + 4) nnz / 2 + 16 N
    in FP64, (4 + 4) nnz / 2 + 8 N in FP32)."""
    import torch
    from goma_gb300 import problem as pb
    from goma_gb300.newton import GomaNewton
    gn = GomaNewton(pb.boussinesq_cube_3d(nel, ra, PR))
    gn.set_ilu_ordering(0)
    gn.set_triangular_solve(0)
    N, nnz = gn.N, gn.nnz
    out = {"workload": "%d^3 Boussinesq cube, one Newton step from rest (Ra %g): ILU(0) in the "
                       "reference's node order, sync-free sweeps, %d GMRES(%d) iterations"
                       % (nel, ra, iters, iters),
           "unknowns": N, "csr_nnz": nnz,
           "bytes": {"spmv_fp64": 12 * nnz + 24 * N, "spmv_fp32": 8 * nnz + 12 * N,
                     "sweep_fp64": 6 * nnz + 16 * N, "sweep_fp32": 4 * nnz + 8 * N}}
    for fp32 in (False, True):
        torch.cuda.synchronize()
        x, conv, st = gn.solve_nonlinear_problem(
            None, residual_tol=1e-300, linear_tol=1e-300, max_newton=1, max_linear_its=iters,
            krylov_dim=iters, fp32_inner=fp32, max_refinements=1, inner_tol=1e-300)
        torch.cuda.synchronize()
        out["fp32" if fp32 else "fp64"] = {
            "linear_its": st["linear_its"], "factor_ms": st["factor_ms"],
            "solve_ms": st["solve_ms"], "ms_per_iteration": st["solve_ms"] / max(1, st["linear_its"])}
        print("krylov:", out["fp32" if fp32 else "fp64"], file=sys.stderr, flush=True)
    gn.close()
    torch.cuda.empty_cache()
    return out


def krylov_step2d(iters=60):
    """The linear-solver kernels on one Newton system of the 96 x 32 Carreau
    step at Re 100 (the state at rest), in the FP32-preconditioner mode:
    a factorisation plus exactly `iters` GMRES(iters) iterations (the
    warp-per-node sweeps of a QUAD9 mesh)."""
    import torch
    from goma_gb300 import problem as pb
    from goma_gb300.newton import GomaNewton
    gn = GomaNewton(pb.carreau_step_2d(96, 32, 100.0))
    gn.set_ilu_ordering(0)
    torch.cuda.synchronize()
    x, conv, st = gn.solve_nonlinear_problem(
        None, residual_tol=1e-300, linear_tol=1e-300, max_newton=1, max_linear_its=iters,
        krylov_dim=iters, fp32_preconditioner=True)
    torch.cuda.synchronize()
    out = {"workload": "96x32 Carreau step, one Newton step from rest (Re 100), FP32 "
                       "preconditioner, %d GMRES(%d) iterations" % (iters, iters),
           "unknowns": gn.N, "linear_its": st["linear_its"], "factor_ms": st["factor_ms"],
           "ms_per_iteration": st["solve_ms"] / max(1, st["linear_its"])}
    gn.close()
    return out


def bfs_continuation(nx=96, ny=32, re0=10.0, re1=800.0, nsteps=200, budget_s=150.0,
                     predictors=("zeroth", "secant", "learned"), krylov=150, fp32=True,
                     warm_steps=75):
    """The learned-predictor configuration: backward-facing step, nx x ny
    QUAD9 Q2/P1, Carreau-Yasuda fluid (mu0 = 1, mu_inf = 0.01, lambda = 1,
    a = 2, n = 0.5), Re re0 -> re1 in nsteps uniform continuation steps, the
    Newton solve to scaled |R| < 1e-10 at every step (FP64 flexible GMRES
    with the ILU(0) in FP32, or plain FP64 with fp32=False).  Each predictor
    runs the same sweep (stopped after budget_s seconds); the network is
    trained with 300 Adam steps at its first training and warm_steps at each
    later one (it carries over between steps).  Reported: steps done, Newton
    and Krylov iterations, wall time and its split, and for the learned run
    the ratio of its guess residual to the secant guess's."""
    import time as _time

    import torch
    from goma_gb300 import problem as pb
    from goma_gb300.continuation import continuation
    from goma_gb300.newton import GomaNewton
    out = {"workload": "backward-facing step %dx%d QUAD9 Q2/P1, Carreau-Yasuda, Re %g -> %g in "
                       "%d steps, scaled |R| < 1e-10, %s" % (
                           nx, ny, re0, re1, nsteps,
                           "FP64 flexible GMRES(%d) with FP32 ILU(0)" % krylov if fp32
                           else "FP64 ILU(0)-GMRES(%d)" % krylov)}
    for pred in predictors:
        gn = GomaNewton(pb.carreau_step_2d(nx, ny, re0))
        opts = dict(residual_tol=1e-10, linear_tol=1e-8, max_newton=25, max_linear_its=3000,
                    krylov_dim=krylov, forcing=1, forcing_max=1e-2, fp32_preconditioner=fp32)
        t0 = _time.perf_counter()
        recs, _ = continuation(gn, re0, re1, nsteps, predictor=pred, newton_opts=opts,
                               learned_opts=dict(steps=300, batch=4096, lr=2e-3,
                                                 warm_steps=warm_steps),
                               time_budget_s=budget_s)
        torch.cuda.synchronize()
        dt = _time.perf_counter() - t0
        res = {"steps_done": len(recs) - 1, "last_re": recs[-1]["lam"], "seconds": dt,
               "newton_its": sum(r["newton_its"] for r in recs[1:]),
               "linear_its": sum(r.get("linear_its", 0) for r in recs[1:]),
               "newton_seconds": sum(r["newton_ms"]["total_ms"] for r in recs[1:]) * 1e-3,
               "predictor_seconds": sum(r.get("predictor_s", 0.0) for r in recs[1:]),
               "candidate_residual_seconds": sum(r.get("residuals_s", 0.0) for r in recs[1:]),
               "training_seconds": sum(r.get("train_s", 0.0) for r in recs[1:]),
               "guesses": {g: sum(1 for r in recs[1:] if r["guess"] == g)
                           for g in ("zeroth", "secant", "learned")}}
        if pred == "learned":
            ratios = [r["candidates"]["learned"] / r["candidates"]["secant"] for r in recs[1:]
                      if "learned" in r.get("candidates", {}) and "secant" in r["candidates"]]
            if ratios:
                res["learned_over_secant_residual"] = {
                    "median": float(np.median(ratios)), "min": float(np.min(ratios)),
                    "max": float(np.max(ratios)), "steps": len(ratios)}
        out[pred] = res
        gn.close()
        torch.cuda.empty_cache()
    return out


def run_reference(args):
    """--impl reference: the reference's CPU assembly of the workload on all
    host threads.  The reference C compiles only where its source tree is
    (oracle/_ref, not on the GPU machine), so the golden-pinned oracle port
    stands in.  Every step is one full nel^3 assembly (zeroing included);
    W untimed steps, then K timed ones; ms_per_step is their mean."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    ca = CpuAssembly(args.nel, threads)
    for _ in range(max(args.warmup, 1)):
        ca.step()
    t = time.perf_counter()
    dts = [ca.step() for _ in range(args.steps)]
    total = time.perf_counter() - t
    ms = 1e3 * total / max(args.steps, 1)
    v = args.nel ** 3 / (ms * 1e-3)
    cb = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
          "sample": ca.describe(args.steps, ms * 1e-3),
          "step_seconds": {"min": min(dts), "max": max(dts)}, "setup_s": ca.setup_s}
    ca.close()
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT,
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(args.nel), "cpu_baseline": cb,
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300")
    ap.add_argument("--nel", type=int, default=NEL)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--path", type=int, default=0,
                    help="element kernel: 0 automatic (4), 1 scalar FP64, 2 FP64 tensor pipe "
                         "with per-fragment coefficients, 3 FP64 tensor-pipe products over "
                         "operand tables, 4 sum factorisation")
    ap.add_argument("--solve-nel", type=int, default=16,
                    help="cube size of the time-to-solve leg (0 skips it; the run with the "
                         "reference's solver settings is added up to 8^3)")
    ap.add_argument("--solve-ilu", type=int, default=-1,
                    help="ILU(0) node order of the time-to-solve leg: 0 the reference's, "
                         "1 multicoloured, -1 by size (multicoloured up to 12^3)")
    ap.add_argument("--solve-modes", default="",
                    help="comma-separated runs of the time-to-solve leg: plain_fp64, "
                         "learned_fp64, learned_fp32, secant_fp32, secant_fp64, "
                         "learned_fp32r, secant_fp32r (FP32 GMRES inside FP64 refinement), "
                         "plain_fp64_reference_solver "
                         "(default: plain_fp64, secant_fp32, learned_fp32)")
    ap.add_argument("--solve-budget", type=float, default=0.0,
                    help="seconds per run of the time-to-solve leg (0: no limit)")
    ap.add_argument("--bfs-budget", type=float, default=150.0,
                    help="seconds per predictor of the bfs workload (the 200-step sweep stops "
                         "there)")
    ap.add_argument("--bfs-fp64", action="store_true",
                    help="the bfs workload's linear solves in FP64 (default: FP64 flexible "
                         "GMRES with the ILU(0) in FP32)")
    ap.add_argument("--bfs-predictors", default="zeroth,secant,learned",
                    help="the bfs workload's predictors, comma separated")
    ap.add_argument("--batch-fp64", action="store_true",
                    help="the batch512_solve workload's linear solves in FP64 (default: FP64 "
                         "flexible GMRES with the ILU(0) in FP32)")
    ap.add_argument("--solve-krylov", type=int, default=300,
                    help="GMRES restart length (Krylov subspace size) of the time-to-solve leg")
    ap.add_argument("--solve-max-linear", type=int, default=4000,
                    help="Krylov iteration limit of one linear solve in the time-to-solve leg")
    ap.add_argument("--solve-inner-tol", type=float, default=1e-3,
                    help="the _fp32r runs' tightest inner GMRES tolerance")
    ap.add_argument("--solve-reuse", type=int, default=0,
                    help="ILU(0) factorisation reuse of the time-to-solve leg: 0 every Newton "
                         "step, 1 once per Newton solve, 2 across solves")
    ap.add_argument("--workloads", default="",
                    help="extra timed workloads, comma separated: reacting (the 64x64x32 "
                         "reacting channel), reacting_small (its 16x16x8 version), batch512 "
                         "(assembly of the 512-problem sweep), batch64_solve (Newton solve of "
                         "64 such problems, n in [16, 32], Re in [10, 100]), batch512_solve "
                         "(the full sweep: 512 problems, n in [16, 64], Re in [10, 1000], Re "
                         "stages of at most 1.6x), bfs (the 96x32 "
                         "Carreau step continuation), ilu_orders (cube solves in both ILU(0) "
                         "node orders, 8^3 to 24^3), cpu_solve (the 8^3 time-to-solve sweep on "
                         "one host core with the oracle's ILU(0)-GMRES(30)), krylovN (the "
                         "linear-solver kernels on one N^3 cube system: factorisation + 30 "
                         "GMRES(30) iterations, FP64 and FP32; krylovNxM: M GMRES(M) "
                         "iterations), krylov_step2d (the same for the 96x32 Carreau step "
                         "in the FP32-preconditioner mode)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)

    import torch
    from goma_gb300 import _lib
    from goma_gb300 import problem as pb
    from goma_gb300.newton import GomaNewton

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    warm = max(args.warmup, 3)
    nel = args.nel

    prob = pb.boussinesq_cube_3d(nel, RA, PR)
    gn = GomaNewton(prob)
    gn.set_assembly_path(args.path)
    kernel_name = {1: "assemble_kernel<3,energy> (scalar FP64)",
                   2: "assemble_tc_kernel<energy> (FP64 DMMA, per-fragment coefficients)",
                   3: "assemble_gemm_kernel<energy> (FP64 DMMA products over operand tables)"}.get(
        args.path, "assemble_sf_kernel<energy> (sum factorisation, FP64)")
    L = gn._L
    N, nnz, msr_len = gn.N, gn.nnz, gn.msr_len
    x_host = gn.dirichlet_init(np.random.default_rng(11).uniform(-1.0, 1.0, N))
    dx = torch.tensor(x_host, dtype=torch.float64, device="cuda")
    dR = torch.empty(N, dtype=torch.float64, device="cuda")
    dv = torch.empty(nnz, dtype=torch.float64, device="cuda")
    # a dedicated (non-default) stream: the library treats a NULL stream as
    # its own stream, so the timing events and the kernels must share this one
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sp = stream.cuda_stream
    assert sp != 0

    def step():
        gn.matrix_fill_full_device(dx.data_ptr(), dR.data_ptr(), dv.data_ptr(), sp)

    for _ in range(warm):
        step()
    torch.cuda.synchronize()
    gn.status()

    # ---- value: device-resident
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler() as clk:
        e0.record(stream)
        for _ in range(args.steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
    gn.status()
    ms = e0.elapsed_time(e1) / args.steps
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
        torch.distributed.barrier()
    elems = prob.mesh.num_elems
    value = world * elems / (ms * 1e-3)

    # ---- e2e: host buffers through the C ABI (x in, R + MSR Jacobian out)
    xh = torch.from_numpy(x_host).pin_memory()
    Rh = torch.empty(N, dtype=torch.float64).pin_memory()
    ah = torch.empty(msr_len, dtype=torch.float64).pin_memory()
    P = lambda t: ctypes.cast(t.data_ptr(), ctypes.POINTER(ctypes.c_double))  # noqa: E731

    def e2e_step():
        _lib.check(L.gb_matrix_fill_full(gn.h, P(xh), P(Rh), P(ah)))

    for _ in range(2):
        e2e_step()
    ke = max(2, min(args.steps, 5))
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    t = time.perf_counter()
    for _ in range(ke):
        e2e_step()
    torch.cuda.synchronize()
    e2e_ms = (time.perf_counter() - t) * 1e3 / ke
    if world > 1:  # the slowest rank's time, as for the device-resident figure
        te = torch.tensor([e2e_ms], device="cuda")
        torch.distributed.all_reduce(te, op=torch.distributed.ReduceOp.MAX)
        e2e_ms = float(te.item())
        torch.distributed.barrier()
    e2e = {"value": world * elems / (e2e_ms * 1e-3), "unit": UNIT,
           "h2d_bytes_per_step": 8 * N, "d2h_bytes_per_step": 8 * N + 8 * msr_len,
           "ms_per_step": e2e_ms,
           "path": "gb_matrix_fill_full: x host->device, R and MSR Jacobian device->host"}

    # ---- roofline of the element kernel
    kms = ctypes.c_double()
    kl = ctypes.c_longlong()
    _lib.check(L.gb_kernel_timing(gn.h, 1, None, None))
    for _ in range(args.steps):
        step()
    torch.cuda.synchronize()
    _lib.check(L.gb_kernel_timing(gn.h, 0, ctypes.byref(kms), ctypes.byref(kl)))
    per_launch_ms = kms.value / max(kl.value, 1)
    elems_per_launch = elems / gn.num_colors
    nloc = 4 * 27 + 4
    dense_flop_el = 2.0 * 27 * nloc * nloc * 4
    flop_el = element_flops(args.path)
    achieved_tf = flop_el * elems_per_launch / (per_launch_ms * 1e-3) / 1e12
    dmma = ctypes.c_double()
    fma = ctypes.c_double()
    dmma_var = ctypes.c_double()
    _lib.check(L.gb_probe_fp64_peaks(ctypes.byref(dmma), ctypes.byref(fma)))
    _lib.check(L.gb_probe_dmma_varying(ctypes.byref(dmma_var)))
    fp64_peak = max(fma.value, dmma_var.value)
    peaks = read_peaks()
    # algorithmic bytes of one launch: its share of the matrix values written,
    # R, x, connectivity and coordinates
    nodes = prob.mesh.num_nodes
    bytes_asm = 8 * nnz + 8 * N + 8 * N + 4 * elems * 27 + 8 * 3 * nodes
    bytes_launch = bytes_asm / gn.num_colors
    hbm_gbs = bytes_launch / (per_launch_ms * 1e-3) / 1e9
    # DRAM traffic of one launch: the 16^3 capture of the same kernel (ncu,
    # one 512-element launch: dram__bytes_read 71.0 MB + write 13.3 MB,
    # profiles/assemble_sf_kernel_hex27_boussinesq.md) scaled by the elements
    # of this launch; the traffic is the matrix update per element, so it
    # grows in proportion
    traffic = (71.0e6 + 13.3e6) / 512 * elems_per_launch if args.path in (0, 4) else None
    roofline = {"bound": "tensor", "achieved": achieved_tf, "peak": fp64_peak,
                "unit": "TFLOP/s", "frac": achieved_tf / fp64_peak,
                "traffic": traffic,
                "traffic_source": "dram__bytes_read.sum + dram__bytes_write.sum of one 512-element "
                                  "launch at 16^3 (ncu), scaled to this launch's elements",
                "kernel": "%s, one colour, %d elements" % (kernel_name, elems_per_launch),
                "launch_ms": per_launch_ms,
                "flop_per_element": flop_el,
                "flop_count": "FP64 operations the kernel's algorithm performs per element "
                              "(FMA = 2), counted term by term",
                "pipe": "FP64 (scalar FMA and mma.sync f64 run at the same rate on GB300)",
                "peak_source": "FP64 throughput measured in-process on this GPU (best of scalar "
                               "FMA chains and mma.sync m8n8k4 f64 with changing operands; "
                               "MEASURED_PEAKS.json has HBM and bf16 only)",
                "fp64_fma_tflops": fma.value, "fp64_dmma_tflops": dmma_var.value,
                "fp64_dmma_constant_operands_tflops": dmma.value,
                "dense_equivalent": {"flop_per_element": dense_flop_el,
                                     "tflops": dense_flop_el * elems_per_launch /
                                     (per_launch_ms * 1e-3) / 1e12,
                                     "note": "2 Q n_loc^2 (d+1): the same Jacobian by dense "
                                             "quadrature-point contractions"},
                "hbm_view": {"achieved_gbs": hbm_gbs, "peak_gbs": peaks.get("hbm_gbs"),
                             "frac": hbm_gbs / peaks.get("hbm_gbs", 6800.0),
                             "bytes_per_launch": bytes_launch}}

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": warm, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": dict(workload_config(nel), unknowns=N, csr_nnz=nnz,
                           colors=gn.num_colors, parallelism="replicas",
                           element_kernel=kernel_name),
            "clocks": clk.summary(), "e2e": e2e, "roofline": roofline,
            "gpu_launches": int(gn.num_colors * args.steps)}
    if rank == 0 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(nel)
    if rank == 0 and args.solve_nel > 0:
        del dv, dx, dR, xh, Rh, ah
        gn.close()
        torch.cuda.empty_cache()
        try:
            line["time_to_solve"] = time_to_solve(
                args.solve_nel, ilu_ordering=args.solve_ilu, reference_solver=args.solve_nel <= 8,
                modes=[m for m in args.solve_modes.split(",") if m] or None,
                budget_s=args.solve_budget or None, factorization_reuse=args.solve_reuse,
                max_linear_its=args.solve_max_linear, krylov=args.solve_krylov,
                inner_tol=args.solve_inner_tol)
        except RuntimeError as exc:   # a continuation step that did not converge
            line["time_to_solve"] = {"error": str(exc)}
    if rank == 0 and args.workloads:
        extra = {}
        for w in args.workloads.split(","):
            if w == "reacting":
                extra[w] = reacting_channel_assembly(64, 64, 32)
            elif w == "reacting_small":
                extra[w] = reacting_channel_assembly(16, 16, 8)
            elif w == "batch512":
                extra[w] = batch_sweep_assembly(512)
            elif w == "batch64_solve":
                extra[w] = batch_sweep_solve(64)
            elif w == "batch512_solve":
                extra[w] = batch_sweep_solve(512, nmin=16, nmax=64, re_max=1000.0,
                                             max_ratio=1.6, budget_s=900.0, check=1,
                                             max_linear_its=2500,
                                             fp32_preconditioner=not args.batch_fp64)
            elif w == "bfs":
                extra[w] = bfs_continuation(budget_s=args.bfs_budget, fp32=not args.bfs_fp64,
                                            predictors=tuple(args.bfs_predictors.split(",")))
            elif w == "ilu_orders":
                extra[w] = ilu_orders()
            elif w == "reuse":
                extra[w] = factorization_reuse_solves(16)
            elif w == "cpu_solve":
                extra[w] = cpu_time_to_solve(8)
            elif w == "reacting_solve":
                extra[w] = reacting_channel_solve()
            elif w == "krylov_step2d":
                extra[w] = krylov_step2d()
            elif w.startswith("krylov"):
                nel_s, _, its_s = w[len("krylov"):].partition("x")
                extra[w] = krylov_kernels(int(nel_s or 16), int(its_s or 30))
        line["workloads"] = extra
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
