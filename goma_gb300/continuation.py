"""Zeroth/first-order parameter continuation with a learned initial guess.

Mirrors continue_problem (src/ac_conti.c:106) for a density (Reynolds
number) sweep of a steady problem:

- ``zeroth``: ALC_ZEROTH, the previous solution is the next guess
  (src/ac_conti.c:759-784);
- ``first``:  ALC_FIRST, x_old + dlambda * dx/dlambda, the tangent from one
  linear solve with the Jacobian at x_old and dR/dlambda by central
  differences of the residual (soln_sens, src/mm_sol_nonlinear.c:3615,
  :3753, :3796);
- ``learned``: a 3 x 256 tanh network (GPU, FP32, trained online by the
  library's own kernels on every converged solution) predicts the fields
  from (x, y[, z], lambda); its guess is used only when its FP64 scaled
  residual is smaller than the fallback's (``zeroth``; ``first`` with
  ``learned+first``), and the Newton solve always decides the answer.

On a failed Newton solve the step is halved and re-predicted
(src/ac_conti.c:986-1045).
"""
import math
import time

import numpy as np

from .newton import GomaNewton


class FieldLayout:
    """Where each unknown lives: nodal velocity components, and the P1
    pressure unknowns at each element's centroid node."""

    def __init__(self, gn: GomaNewton):
        import ctypes

        from . import _lib
        p = gn.problem
        self.dim = p.dim
        nn = p.mesh.num_nodes
        fu = np.empty(nn + 1, np.int32)
        _lib.check(gn._L.gb_first_unknown(gn.h, fu.ctypes.data_as(ctypes.POINTER(ctypes.c_int))))
        self.fu = fu
        self.nvn = p.dim + (1 if p.energy else 0)
        self.centroids = p.mesh.conn[:, 8 if p.dim == 2 else 20]
        self.n_out = self.nvn + p.dim + 1
        # feature scaling: coordinates to [0, 1]
        c = p.mesh.coords
        self.lo = c.min(axis=0)
        self.span = np.maximum(c.max(axis=0) - self.lo, 1e-300)
        self.coords01 = (c - self.lo) / self.span
        cnt = np.diff(fu)
        self.is_cent = cnt > self.nvn

    def targets(self, x):
        """(n_nodes, n_out) targets and mask from an unknown vector."""
        nn = len(self.fu) - 1
        T = np.zeros((nn, self.n_out))
        M = np.zeros((nn, self.n_out), np.float32)
        for a in range(self.nvn):
            T[:, a] = x[self.fu[:-1] + a]
            M[:, a] = 1.0
        cn = np.nonzero(self.is_cent)[0]
        for l in range(self.dim + 1):
            T[cn, self.nvn + l] = x[self.fu[cn] + self.nvn + l]
            M[cn, self.nvn + l] = 1.0
        return T, M

    def assemble(self, Y, N):
        """Unknown vector from (n_nodes, n_out) predictions."""
        x = np.zeros(N)
        for a in range(self.nvn):
            x[self.fu[:-1] + a] = Y[:, a]
        cn = np.nonzero(self.is_cent)[0]
        for l in range(self.dim + 1):
            x[self.fu[cn] + self.nvn + l] = Y[cn, self.nvn + l]
        return x


class LearnedPredictor:
    """(x, y[, z], lambda) -> unknowns at that node, trained online."""

    def __init__(self, gn, lam_range, width=256, hidden=3, seed=0, steps=400, batch=4096,
                 lr=1e-3):
        from .mlp import GpuMLP
        self.lay = FieldLayout(gn)
        self.N = gn.N
        self.net = GpuMLP(self.lay.dim + 1, width, hidden, self.lay.n_out, seed=seed)
        self.lmin, self.lmax = math.log(lam_range[0]), math.log(lam_range[1])
        self.steps, self.batch, self.lr = steps, batch, lr
        self.X, self.T, self.M = [], [], []
        self.tscale = None
        self.trained = 0

    def _features(self, lam):
        s = (math.log(lam) - self.lmin) / max(self.lmax - self.lmin, 1e-300) * 2.0 - 1.0
        c = self.lay.coords01 * 2.0 - 1.0
        return np.hstack([c, np.full((c.shape[0], 1), s)]).astype(np.float32)

    def add(self, lam, x):
        T, M = self.lay.targets(x)
        self.X.append(self._features(lam))
        self.T.append(T)
        self.M.append(M)

    def train(self, seed=0):
        import torch
        X = np.vstack(self.X)
        T = np.vstack(self.T)
        M = np.vstack(self.M)
        # per-output standardisation, refreshed with the data
        mu = (T * M).sum(0) / np.maximum(M.sum(0), 1)
        sd = np.sqrt((((T - mu) * M) ** 2).sum(0) / np.maximum(M.sum(0), 1)) + 1e-12
        self.tscale = (mu, sd)
        Tn = ((T - mu) / sd).astype(np.float32) * M
        dx = torch.tensor(X, device="cuda")
        dt = torch.tensor(Tn, device="cuda")
        dm = torch.tensor(M, device="cuda")
        loss = self.net.train(dx, dt, dm, steps=self.steps, batch=self.batch, lr=self.lr,
                              seed=seed)
        self.trained += 1
        return loss

    def predict(self, lam):
        import torch
        X = torch.tensor(self._features(lam), device="cuda")
        Y = self.net.forward(X).double().cpu().numpy()
        mu, sd = self.tscale
        return self.lay.assemble(Y * sd + mu, self.N)


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


PREDICTORS = ("zeroth", "first", "learned", "learned+first")


def continuation(gn, lam0, lam1, nsteps, predictor="zeroth", x0=None, set_param=_set_density,
                 newton_opts=None, learned_opts=None, spacing="linear", max_halvings=4,
                 verbose=False):
    """Sweep lambda from lam0 to lam1 in nsteps steps (uniform in lambda, or
    in log lambda with spacing="log").  predictor: "zeroth" (ALC_ZEROTH),
    "first" (ALC_FIRST), "learned" (the network, zeroth-order fallback) or
    "learned+first" (the network, first-order fallback).  A step whose
    Newton solve fails is halved and re-predicted from the last converged
    point, at most max_halvings times (src/ac_conti.c:986-1045).  Returns a
    list of per-step records (lambda, guess used, guess residuals, Newton
    iterations, wall time) and the final solution."""
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
                "guess_residual": None, "wall_s": time.perf_counter() - t0}]
    learned = predictor.startswith("learned")
    first = predictor in ("first", "learned+first")
    lp = None
    if learned:
        lp = LearnedPredictor(gn, (min(lam0, lam1), max(lam0, lam1)), **(learned_opts or {}))
        lp.add(lams[0], x)
        lp.train(seed=0)
    lin_keys = ("linear_tol", "fp32_inner", "krylov_dim", "max_linear_its", "inner_tol")
    x_old, lam_old = x, lams[0]
    targets = lams[1:]
    k = 0
    while k < len(targets):
        lam = targets[k]
        t0 = time.perf_counter()
        halvings = 0
        while True:
            cands = {"zeroth": x_old}
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
        if lp is not None:
            lp.add(lam, x)
            if k + 1 < len(targets):
                lp.train(seed=len(records))
        wall = time.perf_counter() - t0
        records.append({"lam": float(lam), "guess": choice, "newton_its": st["newton_its"],
                        "linear_its": st["linear_its"], "guess_residual": res.get(choice),
                        "candidates": res, "halvings": halvings, "wall_s": wall})
        if verbose:
            print(records[-1])
        x_old, lam_old = x, lam
        k += 1
    return records, x
