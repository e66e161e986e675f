"""Parameter continuation with zeroth-order, first-order, secant and learned
initial guesses.

Mirrors continue_problem (src/ac_conti.c:106) for a parameter sweep of a
steady problem (density / Reynolds number, or any parameter set_param sets):

- ``zeroth``: ALC_ZEROTH, the previous solution is the next guess
  (src/ac_conti.c:759-784);
- ``first``:  ALC_FIRST, x_old + dlambda * dx/dlambda, the tangent from one
  linear solve with the Jacobian at x_old and dR/dlambda by central
  differences of the residual (soln_sens, src/mm_sol_nonlinear.c:3615,
  :3753, :3796);
- ``secant``: first-order extrapolation through the last two converged
  solutions (no tangent solve);
- ``learned``: the secant guess plus a curvature correction predicted by a
  3 x 256 tanh network (GPU, FP32, trained online by the library's own
  kernels on the secant errors of the earlier steps).  The plain secant
  guess is the fallback: the learned guess is used only when its FP64
  scaled residual is smaller, and the Newton solve always decides the
  answer;
- ``learned+first``: as ``learned``, with the tangent guess as a third
  candidate.

On a failed Newton solve the step is halved and re-predicted
(src/ac_conti.c:986-1045).
"""
import math
import time

import numpy as np

from .newton import GomaNewton


class FieldLayout:
    """Where each unknown lives: the nodal unknowns (velocity, temperature,
    species) at every node, and the P1 pressure unknowns at each element's
    centroid node."""

    def __init__(self, gn: GomaNewton):
        import ctypes

        from . import _lib
        p = gn.problem
        self.dim = p.dim
        nn = p.mesh.num_nodes
        fu = np.empty(nn + 1, np.int32)
        _lib.check(gn._L.gb_first_unknown(gn.h, fu.ctypes.data_as(ctypes.POINTER(ctypes.c_int))))
        self.fu = fu
        cnt = np.diff(fu)
        self.nvn = int(cnt.min())
        self.n_out = self.nvn + p.dim + 1
        # feature scaling: coordinates to [-1, 1]
        c = p.mesh.coords
        lo = c.min(axis=0)
        span = np.maximum(c.max(axis=0) - lo, 1e-300)
        self.coords11 = (c - lo) / span * 2.0 - 1.0
        self.is_cent = cnt > self.nvn
        self.cn = np.nonzero(self.is_cent)[0]

    def targets(self, x):
        """(n_nodes, n_out) per-node values and their mask from an unknown
        vector (the pressure columns exist at centroid nodes only)."""
        nn = len(self.fu) - 1
        T = np.zeros((nn, self.n_out))
        M = np.zeros((nn, self.n_out), np.float32)
        for a in range(self.nvn):
            T[:, a] = x[self.fu[:-1] + a]
            M[:, a] = 1.0
        for l in range(self.dim + 1):
            T[self.cn, self.nvn + l] = x[self.fu[self.cn] + self.nvn + l]
            M[self.cn, self.nvn + l] = 1.0
        return T, M

    def assemble(self, Y, N):
        """Unknown vector from (n_nodes, n_out) per-node values."""
        x = np.zeros(N)
        for a in range(self.nvn):
            x[self.fu[:-1] + a] = Y[:, a]
        for l in range(self.dim + 1):
            x[self.fu[self.cn] + self.nvn + l] = Y[self.cn, self.nvn + l]
        return x


class LearnedPredictor:
    """Secant predictor plus a learned correction for the curvature of the
    solution path.

    The secant predictor (the cheap first-order predictor, with no tangent
    solve; ALC_FIRST of src/ac_conti.c:759 uses a tangent instead) misses
    the second-order part of x(lambda): its error on a path with curvature
    x''/2 = c is c h (h + h_prev) for a step h after a step h_prev.  A
    network over (x, y[, z], lambda) is trained online, on the GPU by the
    library's own kernels, on the secant errors of every earlier step
    divided by h (h + h_prev) -- samples of the curvature field c -- and the
    guess for the next step is

        x_guess = secant(lam) + h (h + h_prev) * net(coords, lam).

    A fit error in c costs only that fraction of the secant error, so the
    learned guess improves on the secant wherever the curvature field
    carries over from one step to the next."""

    def __init__(self, gn, lam_range, width=256, hidden=3, seed=0, steps=1500, batch=4096,
                 lr=2e-3, log_lambda=False):
        from .mlp import GpuMLP
        self.lay = FieldLayout(gn)
        self.N = gn.N
        self.net = GpuMLP(self.lay.dim + 1, width, hidden, self.lay.n_out, seed=seed)
        self.log_lambda = log_lambda
        self.lmin, self.lmax = self._t(lam_range[0]), self._t(lam_range[1])
        self.steps, self.batch, self.lr = steps, batch, lr
        self.sols = []
        self.X, self.T, self.M = [], [], []
        self.tscale = None
        self.trained = 0

    def _t(self, lam):
        """The sweep variable: lambda, or log lambda for a sweep uniform in
        log lambda."""
        return math.log(lam) if self.log_lambda else float(lam)

    def _features(self, t):
        s = (t - self.lmin) / max(self.lmax - self.lmin, 1e-300) * 2.0 - 1.0
        c = self.lay.coords11
        return np.hstack([c, np.full((c.shape[0], 1), s)]).astype(np.float32)

    def secant(self, lam):
        """First-order extrapolation through the last two recorded solutions
        (the last solution itself while only one is known)."""
        t = self._t(lam)
        tk, xk = self.sols[-1]
        if len(self.sols) < 2:
            return xk.copy()
        tp, xp = self.sols[-2]
        return xk + (t - tk) * (xk - xp) / (tk - tp)

    def _hh(self, t):
        tk = self.sols[-1][0]
        tp = self.sols[-2][0]
        h, hp = t - tk, tk - tp
        return h * (h + hp)

    def add(self, lam, x):
        """Record a converged solution; once two earlier ones are known, the
        secant predictor's error at this one becomes a training sample."""
        t = self._t(lam)
        x = np.array(x, np.float64)
        if len(self.sols) >= 2:
            hh = self._hh(t)
            if hh != 0.0:
                T, M = self.lay.targets((x - self.secant(lam)) / hh)
                self.X.append(self._features(t))
                self.T.append(T)
                self.M.append(M)
        self.sols.append((t, x))

    @property
    def ready(self):
        return bool(self.X)

    def train(self, seed=0):
        import torch
        if not self.X:
            return None
        X = np.vstack(self.X)
        T = np.vstack(self.T)
        M = np.vstack(self.M)
        # per-output standardisation, refreshed with the data
        mu = (T * M).sum(0) / np.maximum(M.sum(0), 1)
        sd = np.sqrt((((T - mu) * M) ** 2).sum(0) / np.maximum(M.sum(0), 1))
        sd = np.where(sd > 0, sd, 1.0)
        self.tscale = (mu, sd)
        Tn = ((T - mu) / sd).astype(np.float32) * M
        dx = torch.tensor(X, device="cuda")
        dt = torch.tensor(Tn, device="cuda")
        dm = torch.tensor(M, device="cuda")
        # Adam at the given rate, then a quarter as many steps at a tenth of it
        self.net.train(dx, dt, dm, steps=self.steps, batch=self.batch, lr=self.lr, seed=seed)
        loss = self.net.train(dx, dt, dm, steps=max(self.steps // 4, 1), batch=self.batch,
                              lr=0.1 * self.lr, seed=seed + 7919)
        self.trained += 1
        return loss

    def curvature(self, lam):
        """The network's curvature field at lam, as an unknown vector."""
        import torch
        X = torch.tensor(self._features(self._t(lam)), device="cuda")
        Y = self.net.forward(X).double().cpu().numpy()
        mu, sd = self.tscale
        return self.lay.assemble(Y * sd + mu, self.N)

    def predict(self, lam):
        return self.secant(lam) + self._hh(self._t(lam)) * self.curvature(lam)


def _set_density(gn, rho):
    m = gn.problem.material
    m.density = rho
    gn.set_material(m)


def scaled_residual_l2(gn, x):
    """L2 norm of the row-sum-scaled FP64 residual at x (the quantity the
    Newton loop tests, src/mm_sol_nonlinear.c:1451)."""
    import torch
    dx = torch.tensor(x, dtype=torch.float64, device="cuda")
    dR = torch.empty(gn.N, dtype=torch.float64, device="cuda")
    dv = torch.empty(gn.nnz, dtype=torch.float64, device="cuda")
    gn.matrix_fill_full_device(dx.data_ptr(), dR.data_ptr(), dv.data_ptr(), None)
    gn.status()
    gn.scale_device(dv.data_ptr(), dR.data_ptr())
    torch.cuda.synchronize()
    return float(torch.linalg.vector_norm(dR).item())


def tangent(gn, x, lam, set_param, rel=1e-6, **solve_opts):
    """dx/dlambda at (x, lam): J dx/dlambda = -dR/dlambda, central
    differences in lambda (soln_sens, src/mm_sol_nonlinear.c:3615)."""
    import torch
    N = gn.N
    h = rel * max(abs(lam), 1.0)
    dx = torch.tensor(x, dtype=torch.float64, device="cuda")
    Rp = torch.empty(N, dtype=torch.float64, device="cuda")
    Rm = torch.empty(N, dtype=torch.float64, device="cuda")
    set_param(gn, lam + h)
    gn.matrix_fill_full_device(dx.data_ptr(), Rp.data_ptr(), None, None)
    set_param(gn, lam - h)
    gn.matrix_fill_full_device(dx.data_ptr(), Rm.data_ptr(), None, None)
    set_param(gn, lam)
    R0 = torch.empty(N, dtype=torch.float64, device="cuda")
    dv = torch.empty(gn.nnz, dtype=torch.float64, device="cuda")
    gn.matrix_fill_full_device(dx.data_ptr(), R0.data_ptr(), dv.data_ptr(), None)
    gn.status()
    scale = torch.empty(N, dtype=torch.float64, device="cuda")
    gn.scale_device(dv.data_ptr(), R0.data_ptr(), scale.data_ptr())
    torch.cuda.synchronize()
    rhs = -((Rp - Rm) / (2.0 * h)) / scale
    sens = torch.empty(N, dtype=torch.float64, device="cuda")
    gn.linear_solve_device(dv.data_ptr(), rhs.data_ptr(), sens.data_ptr(), **solve_opts)
    return sens.cpu().numpy()


PREDICTORS = ("zeroth", "first", "secant", "learned", "learned+first")


def continuation(gn, lam0, lam1, nsteps, predictor="zeroth", x0=None, set_param=_set_density,
                 newton_opts=None, learned_opts=None, spacing="linear", max_halvings=4,
                 verbose=False):
    """Sweep lambda from lam0 to lam1 in nsteps steps (uniform in lambda, or
    in log lambda with spacing="log").  predictor: "zeroth" (ALC_ZEROTH),
    "first" (ALC_FIRST), "secant", "learned" (secant + the network's
    curvature correction, secant fallback) or "learned+first" (the same
    with the tangent guess as another candidate).  Among several candidate
    guesses the one with the smallest FP64 scaled residual is used.  A step
    whose Newton solve fails is halved and re-predicted from the last
    converged point, at most max_halvings times (src/ac_conti.c:986-1045).
    Returns a list of per-step records (lambda, guess used, candidate
    residuals, Newton iterations, wall time) and the final solution."""
    if predictor not in PREDICTORS:
        raise ValueError("predictor must be one of %s" % (PREDICTORS,))
    newton_opts = dict(newton_opts or {})
    if spacing == "log":
        lams = list(np.exp(np.linspace(math.log(lam0), math.log(lam1), nsteps + 1)))
    else:
        lams = list(np.linspace(lam0, lam1, nsteps + 1))
    set_param(gn, lams[0])
    t0 = time.perf_counter()
    x, conv, st = gn.solve_nonlinear_problem(x0, **newton_opts)
    if not conv:
        raise RuntimeError("first continuation step did not converge")
    records = [{"lam": float(lams[0]), "guess": "initial", "newton_its": st["newton_its"],
                "linear_its": st["linear_its"], "guess_residual": None,
                "wall_s": time.perf_counter() - t0,
                "newton_ms": {k2: st[k2] for k2 in ("assemble_ms", "scale_ms", "factor_ms",
                                                    "solve_ms", "total_ms")}}]
    learned = predictor.startswith("learned")
    first = predictor in ("first", "learned+first")
    secant = predictor == "secant" or learned
    lp = None
    if learned:
        lp = LearnedPredictor(gn, (min(lam0, lam1), max(lam0, lam1)),
                              log_lambda=(spacing == "log"), **(learned_opts or {}))
        lp.add(lams[0], x)
    hist = [(lams[0], x)]
    lin_keys = ("linear_tol", "fp32_inner", "krylov_dim", "max_linear_its", "inner_tol")
    x_old, lam_old = x, lams[0]
    targets = lams[1:]
    k = 0
    while k < len(targets):
        lam = targets[k]
        t0 = time.perf_counter()
        halvings = 0
        while True:
            cands = {}
            if secant and len(hist) >= 2:
                (lp_, xp_), (lk_, xk_) = hist[-2], hist[-1]
                if spacing == "log":
                    ht, hp = math.log(lam) - math.log(lk_), math.log(lk_) - math.log(lp_)
                else:
                    ht, hp = lam - lk_, lk_ - lp_
                cands["secant"] = xk_ + (ht / hp) * (xk_ - xp_)
            else:
                cands["zeroth"] = x_old
            if first:
                sens = tangent(gn, x_old, lam_old, set_param,
                               **{k2: v for k2, v in newton_opts.items() if k2 in lin_keys})
                cands["first"] = x_old + (lam - lam_old) * sens
            set_param(gn, lam)
            if learned and lp.trained:
                cands["learned"] = gn.dirichlet_init(lp.predict(lam))
            res = {}
            if len(cands) > 1:
                for name, xc in cands.items():
                    res[name] = scaled_residual_l2(gn, xc)
                choice = min(res, key=lambda n: (res[n] if np.isfinite(res[n]) else np.inf))
            else:
                choice = next(iter(cands))
            guess = gn.dirichlet_init(cands[choice])
            x, conv, st = gn.solve_nonlinear_problem(guess, **newton_opts)
            if conv:
                break
            if halvings >= max_halvings:
                raise RuntimeError("continuation step at lambda=%g did not converge" % lam)
            halvings += 1
            lam = 0.5 * (lam_old + lam)
            targets.insert(k, lam)
        hist.append((lam, x))
        if lp is not None:
            lp.add(lam, x)
            if k + 1 < len(targets) and lp.ready:
                lp.train(seed=len(records))
        wall = time.perf_counter() - t0
        records.append({"lam": float(lam), "guess": choice, "newton_its": st["newton_its"],
                        "linear_its": st["linear_its"], "guess_residual": res.get(choice),
                        "candidates": res, "halvings": halvings, "wall_s": wall,
                        "newton_ms": {k2: st[k2] for k2 in ("assemble_ms", "scale_ms",
                                                            "factor_ms", "solve_ms",
                                                            "total_ms")}})
        if verbose:
            print(records[-1])
        x_old, lam_old = x, lam
        k += 1
    return records, x
