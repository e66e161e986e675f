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
- ``learned``: the secant guess with a correction of the rate of change
  predicted, unknown by unknown, by a 3 x 256 tanh network from the recent
  rate history (GPU, FP32, trained online by the library's own kernels on
  the earlier steps of the sweep).  The plain secant guess is the
  fallback: the learned guess is used only when its FP64 scaled residual
  is smaller, and the Newton solve always decides the answer;
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
    """Where each unknown lives: its node and its position in the node's
    block of unknowns (the nodal fields, then at centroid nodes the P1
    pressures)."""

    def __init__(self, gn: GomaNewton):
        import ctypes

        from . import _lib
        p = gn.problem
        self.dim = p.dim
        nn = p.mesh.num_nodes
        fu = np.empty(nn + 1, np.int32)
        _lib.check(gn._L.gb_first_unknown(gn.h, fu.ctypes.data_as(ctypes.POINTER(ctypes.c_int))))
        cnt = np.diff(fu)
        self.N = int(fu[-1])
        self.nfield = int(cnt.max())
        self.node = np.repeat(np.arange(nn), cnt)
        self.field = np.arange(self.N) - np.repeat(fu[:-1], cnt)
        c = p.mesh.coords
        lo = c.min(axis=0)
        span = np.maximum(c.max(axis=0) - lo, 1e-300)
        self.coords11 = ((c - lo) / span * 2.0 - 1.0)[self.node]


class LearnedPredictor:
    """Learned extrapolation along the sweep, one unknown at a time.

    For every unknown the network sees the rate of change of the last step
    r1 = (x_k - x_{k-1}) / h1, how that rate changed over the step before,
    (r1 - r2) (h + h1) / (h1 + h2), which field it belongs to and where its
    node is, and predicts the change of the rate over the next step,
    r - r1.  The guess is the secant guess corrected by it:

        x_guess = x_k + h (r1 + net(...)).

    A zero network is the secant predictor (the cheap first-order
    predictor, with no tangent solve; ALC_FIRST of src/ac_conti.c:759 uses a
    tangent instead), and a network that answers the rate change itself is
    quadratic extrapolation; trained online (on the GPU, by the library's
    own kernels) on every earlier step of the sweep, it learns how the
    rates of this problem's fields actually evolve.  Inputs and targets are
    scaled per field by the RMS of r1."""

    def __init__(self, gn, lam_range, width=256, hidden=3, seed=0, steps=1500, batch=4096,
                 lr=2e-3, log_lambda=False, warm_steps=None):
        from .mlp import GpuMLP
        self.lay = FieldLayout(gn)
        self.N = gn.N
        self.n_in = 2 + self.lay.nfield + self.lay.dim
        self.net = GpuMLP(self.n_in, width, hidden, 1, seed=seed)
        self.log_lambda = log_lambda
        self.steps, self.batch, self.lr = steps, batch, lr
        # the network carries over from one continuation step to the next:
        # after the first training, warm_steps Adam steps (default: steps)
        self.warm_steps = steps if warm_steps is None else warm_steps
        self.sols = []
        self.X, self.T = [], []
        self.trained = 0

    def _t(self, lam):
        """The sweep variable: lambda, or log lambda for a sweep uniform in
        log lambda."""
        return math.log(lam) if self.log_lambda else float(lam)

    def _sigma(self, r1):
        f = self.lay.field
        ms = np.bincount(f, weights=r1 * r1, minlength=self.lay.nfield)
        n = np.maximum(np.bincount(f, minlength=self.lay.nfield), 1)
        s = np.sqrt(ms / n)
        return np.where(s > 0, s, 1.0)[f]

    def _features(self, r1, dr, sig):
        lay = self.lay
        X = np.zeros((self.N, self.n_in), np.float32)
        X[:, 0] = r1 / sig
        X[:, 1] = dr / sig
        X[np.arange(self.N), 2 + lay.field] = 1.0
        X[:, 2 + lay.nfield:] = lay.coords11
        return X

    def _history(self, t_next, upto):
        """Rates r1, r2 and the scaled rate change for predicting the step to
        t_next from the first `upto` recorded solutions."""
        (t2, x2), (t1, x1), (t0, x0) = self.sols[upto - 3], self.sols[upto - 2], self.sols[upto - 1]
        h1, h2, h = t0 - t1, t1 - t2, t_next - t0
        r1 = (x0 - x1) / h1
        r2 = (x1 - x2) / h2
        return r1, (r1 - r2) * (h + h1) / (h1 + h2), h

    def add(self, lam, x):
        """Record a converged solution; once three earlier ones are known, the
        step to this one becomes a training sample (a row per unknown)."""
        t = self._t(lam)
        x = np.array(x, np.float64)
        if len(self.sols) >= 3:
            r1, dr, h = self._history(t, len(self.sols))
            sig = self._sigma(r1)
            r = (x - self.sols[-1][1]) / h
            self.X.append(self._features(r1, dr, sig))
            self.T.append(((r - r1) / sig).astype(np.float32)[:, None])
        self.sols.append((t, x))

    @property
    def ready(self):
        return bool(self.X)

    def train(self, seed=0):
        import torch
        if not self.X:
            return None
        # the training set stays on the device; only the samples added since
        # the last training are copied (a sweep's set grows by N rows a step)
        n_dev = getattr(self, "_n_dev", 0)
        if n_dev < len(self.X):
            nx = torch.tensor(np.vstack(self.X[n_dev:]), device="cuda")
            nt = torch.tensor(np.vstack(self.T[n_dev:]), device="cuda")
            self._dX = nx if n_dev == 0 else torch.cat([self._dX, nx])
            self._dT = nt if n_dev == 0 else torch.cat([self._dT, nt])
            self._dM = torch.ones_like(self._dT)
            self._n_dev = len(self.X)
        dx, dt, dm = self._dX, self._dT, self._dM
        # Adam at the given rate, then a quarter as many steps at a tenth of it
        steps = self.steps if self.trained == 0 else self.warm_steps
        self.net.train(dx, dt, dm, steps=steps, batch=self.batch, lr=self.lr, seed=seed)
        loss = self.net.train(dx, dt, dm, steps=max(steps // 4, 1), batch=self.batch,
                              lr=0.1 * self.lr, seed=seed + 7919)
        self.trained += 1
        return loss

    def predict(self, lam):
        import torch
        t = self._t(lam)
        r1, dr, h = self._history(t, len(self.sols))
        sig = self._sigma(r1)
        X = torch.tensor(self._features(r1, dr, sig), device="cuda")
        corr = self.net.forward(X).cpu().numpy()[:, 0].astype(np.float64) * sig
        return self.sols[-1][1] + h * (r1 + corr)


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
    return float(np.linalg.norm(dR.cpu().numpy()))


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
                 verbose=False, time_budget_s=None):
    """Sweep lambda from lam0 to lam1 in nsteps steps (uniform in lambda, or
    in log lambda with spacing="log").  predictor: "zeroth" (ALC_ZEROTH),
    "first" (ALC_FIRST), "secant", "learned" (secant + the network's
    rate correction, secant fallback) or "learned+first" (the same
    with the tangent guess as another candidate).  Among several candidate
    guesses the one with the smallest FP64 scaled residual is used.  A step
    whose Newton solve fails is halved and re-predicted from the last
    converged point, at most max_halvings times (src/ac_conti.c:986-1045).
    With time_budget_s the sweep stops after the first step that ends past
    that many seconds.  Returns a list of per-step records (lambda, guess
    used, candidate residuals, Newton iterations, wall time) and the last
    solution."""
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
                "linear_its": st["linear_its"], "factorizations": st["factorizations"],
                "guess_residual": None,
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
    lin_keys = ("linear_tol", "fp32_inner", "fp32_preconditioner", "krylov_dim", "max_linear_its",
                "inner_tol")
    x_old, lam_old = x, lams[0]
    targets = lams[1:]
    k = 0
    t_sweep = time.perf_counter()
    while k < len(targets):
        if time_budget_s is not None and time.perf_counter() - t_sweep > time_budget_s:
            break
        lam = targets[k]
        t0 = time.perf_counter()
        halvings = 0
        pred_s = cand_s = res_s = 0.0
        while True:
            tp = time.perf_counter()
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
            tr = time.perf_counter()
            cand_s += tr - tp
            res = {}
            if len(cands) > 1:
                for name, xc in cands.items():
                    res[name] = scaled_residual_l2(gn, xc)
                choice = min(res, key=lambda n: (res[n] if np.isfinite(res[n]) else np.inf))
            else:
                choice = next(iter(cands))
            guess = gn.dirichlet_init(cands[choice])
            res_s += time.perf_counter() - tr
            pred_s += time.perf_counter() - tp
            x, conv, st = gn.solve_nonlinear_problem(guess, **newton_opts)
            if conv:
                break
            if halvings >= max_halvings:
                raise RuntimeError("continuation step at lambda=%g did not converge" % lam)
            halvings += 1
            lam = 0.5 * (lam_old + lam)
            targets.insert(k, lam)
        hist.append((lam, x))
        train_s = 0.0
        if lp is not None:
            tt = time.perf_counter()
            lp.add(lam, x)
            if k + 1 < len(targets) and lp.ready:
                lp.train(seed=len(records))
            train_s = time.perf_counter() - tt
        wall = time.perf_counter() - t0
        records.append({"lam": float(lam), "guess": choice, "newton_its": st["newton_its"],
                        "linear_its": st["linear_its"], "factorizations": st["factorizations"],
                        "guess_residual": res.get(choice),
                        "candidates": res, "halvings": halvings, "wall_s": wall,
                        "predictor_s": pred_s, "candidates_s": cand_s, "residuals_s": res_s,
                        "train_s": train_s,
                        "newton_ms": {k2: st[k2] for k2 in ("assemble_ms", "scale_ms",
                                                            "factor_ms", "solve_ms",
                                                            "total_ms")}})
        if verbose:
            print(records[-1])
        x_old, lam_old = x, lam
        k += 1
    return records, x
