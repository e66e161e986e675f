"""Pseudo-arclength continuation: solution branches followed through turning
points, where a continuation in the parameter itself (continuation.py)
must stop.

The reference reaches turning points through LOCA's arc-length
continuation (src/loca_lib.c:717, arc_length_continuation).  This is
Keller's pseudo-arclength method with the bordering algorithm:

    the unknowns are (x, lam); the equations R(x, lam) = 0 and
        N = theta/n * xdot^T (x - x_k) + lamdot (lam - lam_k) - ds = 0,
    with (xdot, lamdot) the unit tangent at the last point (x_k, lam_k).
    A Newton step solves the bordered system by two solves with J:
        J a = -R,  J b = -dR/dlam  (central differences in lam),
        dlam = -(N + theta/n xdot^T a) / (lamdot + theta/n xdot^T b),
        dx = a + dlam b.

The predictor steps ds along the tangent; the next tangent is (b, 1)
normalised and oriented along the previous one, so the branch is followed
around a fold.  A corrector that fails halves ds; quick convergence grows
it up to ds_max.

The driver needs a linearisation callback, linearize(x, lam) ->
(R, solve, scale): the (row-scaled) residual, a function solving J dx =
rhs for the same scaling, and the row scales to apply to other residuals.
`GomaArcProblem` provides it from the library's host calls
(gb_matrix_fill_full, row-sum scaling as row_sum_scaling_scale does it,
gb_linear_solve).
"""
import math

import numpy as np


# array helpers: the driver runs on numpy arrays (host problems) or torch
# tensors (GomaArcProblemDevice, vectors resident on the GPU)
def _dot(a, b):
    return float((a * b).sum())


def _norm(a):
    return math.sqrt(_dot(a, a))


def _finite(a):
    if isinstance(a, np.ndarray):
        return bool(np.all(np.isfinite(a)))
    import torch
    return bool(torch.isfinite(a).all())


def _copy(a):
    return a.copy() if isinstance(a, np.ndarray) else a.clone()


def msr_row_scale(ija, a):
    """Row scales of an MSR matrix as the reference's row_sum_scale_MSR
    (src/sl_matrix_util.c:506): sign(a_ii) * sum_j |a_ij| (1 for an
    all-zero row); returns (scaled copy of a, scales)."""
    ija = np.asarray(ija, np.int64)
    N = int(ija[0]) - 1
    off = np.abs(a[N + 1:ija[N]])
    counts = np.diff(ija[:N + 1])
    rows = np.repeat(np.arange(N), counts)
    s = np.abs(a[:N]).copy()
    np.add.at(s, rows, off)
    neg = (np.abs(a[:N]) > 1e-200) & (a[:N] < 0.0)
    s[neg] = -s[neg]
    s[s == 0.0] = 1.0
    out = a.copy()
    out[:N] /= s
    out[N + 1:ija[N]] /= s[rows]
    return out, s


class GomaArcProblem:
    """linearize() for a library context: assembly through
    gb_matrix_fill_full, the reference's row-sum scaling, ILU(0)-GMRES
    through gb_linear_solve (options as for the Newton solve)."""

    def __init__(self, gn, set_param, **linear_opts):
        self.gn = gn
        self.set_param = set_param
        self.ija = gn.msr_pattern()
        self.opts = dict(linear_tol=1e-10, max_linear_its=4000, krylov_dim=60)
        self.opts.update(linear_opts)

    def residual(self, x, lam):
        self.set_param(self.gn, lam)
        R, _ = self.gn.matrix_fill_full(x, jacobian=False)
        return R

    def linearize(self, x, lam):
        self.set_param(self.gn, lam)
        R, a = self.gn.matrix_fill_full(x)
        a_s, s = msr_row_scale(self.ija, a)

        def solve(rhs):
            dx, _, _ = self.gn.linear_solve(a_s, rhs, **self.opts)
            return dx

        return R / s, solve, s

    def dirichlet_init(self, x):
        return self.gn.dirichlet_init(x)


class GomaArcProblemDevice:
    """linearize() with every vector on the GPU (torch float64 tensors):
    assembly through gb_matrix_fill_full_device into the context's CSR
    values, row-sum scaling on the device (gb_row_sum_scale_device), and
    ILU(0)-GMRES through gb_linear_solve_device, factorising once per
    linearisation and reusing the factors for its further right-hand sides.
    Only scalars (norms, dot products) come back to the host."""

    def __init__(self, gn, set_param, **linear_opts):
        import torch
        self.gn = gn
        self.set_param = set_param
        self.opts = dict(linear_tol=1e-10, max_linear_its=4000, krylov_dim=60)
        self.opts.update(linear_opts)
        self.torch = torch
        dev = torch.device("cuda")
        self.R = torch.empty(gn.N, dtype=torch.float64, device=dev)
        self.scale = torch.empty(gn.N, dtype=torch.float64, device=dev)

    def _sync(self):
        self.gn.status()   # the library stream: its assembly / scaling are done

    def residual(self, x, lam):
        self.set_param(self.gn, lam)
        self.torch.cuda.current_stream().synchronize()
        self.gn.matrix_fill_full_device(x.data_ptr(), self.R.data_ptr(), None)
        self._sync()
        return self.R.clone()

    def linearize(self, x, lam):
        torch = self.torch
        self.set_param(self.gn, lam)
        torch.cuda.current_stream().synchronize()
        gn = self.gn
        gn.matrix_fill_full_device(x.data_ptr(), self.R.data_ptr(), gn.d_vals)
        gn.scale_device(gn.d_vals, self.R.data_ptr(), self.scale.data_ptr())
        self._sync()
        R = self.R.clone()
        scale = self.scale.clone()
        first = [True]

        def solve(rhs):
            rhs = rhs.contiguous()
            dx = torch.empty_like(rhs)
            torch.cuda.current_stream().synchronize()
            gn.linear_solve_device(gn.d_vals, rhs.data_ptr(), dx.data_ptr(),
                                   factorization_reuse=0 if first[0] else 2, **self.opts)
            first[0] = False
            return dx

        return R, solve, scale

    def dirichlet_init(self, x):
        return self.gn.dirichlet_init(x)


def arclength_continuation(problem, x0, lam0, ds, nsteps, lam_bounds=None, theta=1.0,
                           tol=1e-10, max_corrector=12, ds_min=None, ds_max=None,
                           dlam_rel=1e-6, direction=1.0):
    """Follows the branch through (x0, lam0) (x0 a converged solution) for
    nsteps pseudo-arclength steps of initial length ds, stopping early when
    lam leaves lam_bounds (lo, hi).  `problem` provides residual(x, lam)
    and linearize(x, lam) (see the module docstring).  direction +1 starts
    towards increasing lam.  Returns a list of records (lam, step length,
    corrector iterations, residual norm, lam component of the tangent) and
    the list of solutions."""
    ds_min = ds_min if ds_min is not None else ds / 64.0
    ds_max = ds_max if ds_max is not None else ds * 8.0
    x = _copy(x0) if not isinstance(x0, np.ndarray) else np.asarray(x0, np.float64).copy()
    lam = float(lam0)
    n = x.numel() if hasattr(x, "numel") else x.size
    w = theta / n

    def dR_dlam(xc, lc, scale):
        h = dlam_rel * max(abs(lc), 1.0)
        return (problem.residual(xc, lc + h) - problem.residual(xc, lc - h)) / (2.0 * h) / scale

    def tangent(xc, lc, prev):
        _, solve, scale = problem.linearize(xc, lc)
        b = solve(-dR_dlam(xc, lc, scale))
        norm = math.sqrt(w * _dot(b, b) + 1.0)
        t = (b / norm, 1.0 / norm)
        if prev is not None:
            if w * _dot(t[0], prev[0]) + t[1] * prev[1] < 0.0:
                t = (-t[0], -t[1])
        elif direction < 0:
            t = (-t[0], -t[1])
        return t

    t = tangent(x, lam, None)
    records = [{"lam": lam, "ds": 0.0, "corrector_its": 0, "residual": None,
                "lamdot": t[1]}]
    sols = [_copy(x)]
    step = 0
    while step < nsteps:
        xp = x + ds * t[0]
        lp = lam + ds * t[1]
        xc, lc = xp, lp
        ok = False
        rn = np.inf
        for it in range(1, max_corrector + 1):
            R, solve, scale = problem.linearize(xc, lc)
            rn = _norm(R)
            Nc = w * _dot(t[0], xc - x) + t[1] * (lc - lam) - ds
            if rn < tol and abs(Nc) < tol * max(1.0, abs(ds)):
                ok = True
                break
            a = solve(-R)
            b = solve(-dR_dlam(xc, lc, scale))
            dl = -(Nc + w * _dot(t[0], a)) / (t[1] + w * _dot(t[0], b))
            xc = xc + a + dl * b
            lc = lc + dl
            if not _finite(xc):
                break
        if not ok:
            ds *= 0.5
            if abs(ds) < ds_min:
                raise RuntimeError("arc-length step fell below ds_min at lam=%g" % lam)
            continue
        x, lam = xc, lc
        t = tangent(x, lam, t)
        records.append({"lam": lam, "ds": ds, "corrector_its": it, "residual": rn,
                        "lamdot": t[1]})
        sols.append(_copy(x))
        step += 1
        if it <= 3:
            ds = min(ds * 1.5, ds_max)
        if lam_bounds is not None and not (lam_bounds[0] <= lam <= lam_bounds[1]):
            break
    return records, sols
