"""Host-side mirror of the reference interface for the Newton path.

``GomaNewton`` wraps one problem context of libgbnewton.so and exposes the
calls a Goma maintainer would bind: the MSR pattern of
alloc_MSR_sparse_arrays, matrix_fill_full, and (in later layers) the linear
solve and solve_nonlinear_problem.  Host arrays are numpy; device arrays
are raw pointers (e.g. ``torch.Tensor.data_ptr()``).
"""
import ctypes

import numpy as np

from . import _lib
from .problem import make_desc


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def msr_pattern_host(problem):
    """The reference's MSR ija for a problem, computed on the host only."""
    L = _lib.load()
    desc, keep = make_desc(problem)
    n = ctypes.c_longlong()
    _lib.check(L.gb_msr_pattern_host(ctypes.byref(desc), None, ctypes.byref(n)))
    ija = np.empty(n.value, np.int32)
    _lib.check(L.gb_msr_pattern_host(ctypes.byref(desc), ija.ctypes.data_as(
        ctypes.POINTER(ctypes.c_int)), ctypes.byref(n)))
    del keep
    return ija


class GomaNewton:
    """One Q2/P1 problem resident on the GPU."""

    def __init__(self, problem):
        self.problem = problem
        self._L = _lib.load()
        desc, keep = make_desc(problem)
        h = ctypes.c_void_p()
        _lib.check(self._L.gb_create(ctypes.byref(desc), ctypes.byref(h)))
        self.h = h
        del keep
        self.N = self._L.gb_num_unknowns(self.h)
        self.msr_len = self._L.gb_msr_length(self.h)
        self.nnz = self._L.gb_csr_nnz(self.h)
        self.num_colors = self._L.gb_num_colors(self.h)
        x, R, v, rp, ci = (ctypes.c_void_p() for _ in range(5))
        _lib.check(self._L.gb_device_buffers(self.h, ctypes.byref(x), ctypes.byref(R),
                                             ctypes.byref(v), ctypes.byref(rp), ctypes.byref(ci)))
        self.d_x, self.d_R, self.d_vals = x.value, R.value, v.value
        self.d_rowptr, self.d_colidx = rp.value, ci.value
        self.stream = self._L.gb_stream(self.h)

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self._L.gb_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # --- setup queries
    def msr_pattern(self):
        ija = np.empty(self.msr_len, np.int32)
        _lib.check(self._L.gb_msr_pattern(self.h, ija.ctypes.data_as(
            ctypes.POINTER(ctypes.c_int))))
        return ija

    def csr_pattern(self):
        rp = np.empty(self.N + 1, np.int64)
        ci = np.empty(self.nnz, np.int32)
        _lib.check(self._L.gb_csr_pattern(self.h, rp.ctypes.data_as(
            ctypes.POINTER(ctypes.c_longlong)), ci.ctypes.data_as(ctypes.POINTER(ctypes.c_int))))
        return rp, ci

    def csr_row(self, d_vals, row):
        """(64-bit start offset, columns, values) of one CSR row of the device
        values d_vals (gb_csr_row)."""
        start = ctypes.c_longlong()
        n = self._L.gb_csr_row(self.h, None, int(row), ctypes.byref(start), None, None, 0)
        if n < 0:
            _lib.check(-1)
        cols = np.empty(n, np.int32)
        vals = np.empty(n)
        if self._L.gb_csr_row(self.h, d_vals, int(row), ctypes.byref(start),
                              cols.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), _dp(vals), n) != n:
            _lib.check(-1)
        return start.value, cols, vals

    def dirichlet_init(self, x):
        x = np.ascontiguousarray(x, np.float64).copy()
        _lib.check(self._L.gb_dirichlet_init(self.h, _dp(x)))
        return x

    def set_ilu_ordering(self, ordering):
        """ILU(0) node order of later solves: 0 the reference's, 1 multicoloured."""
        _lib.check(self._L.gb_set_ilu_ordering(self.h, int(ordering)))

    def set_element_density(self, rho):
        """Per-element densities (None: the material's) for later assemblies."""
        if rho is None:
            _lib.check(self._L.gb_set_element_density(self.h, None))
            return
        rho = np.ascontiguousarray(rho, np.float64)
        if rho.shape != (self.problem.mesh.num_elems,):
            raise ValueError("one density per element")
        _lib.check(self._L.gb_set_element_density(self.h, _dp(rho)))

    # --- matrix_fill_full
    def matrix_fill_full(self, x, jacobian=True):
        """Host arrays in and out: returns (R, a_msr or None)."""
        x = np.ascontiguousarray(x, np.float64)
        R = np.empty(self.N)
        a = np.empty(self.msr_len) if jacobian else None
        _lib.check(self._L.gb_matrix_fill_full(self.h, _dp(x), _dp(R),
                                               _dp(a) if a is not None else None))
        return R, a

    def matrix_fill_full_transient(self, x, xdot, delta_t, theta, jacobian=True):
        """Transient matrix_fill_full (host arrays): the mass terms of xdot
        and their (1 + 2 theta) / delta_t sensitivity.  (R, a_msr or None)."""
        x = np.ascontiguousarray(x, np.float64)
        xdot = np.ascontiguousarray(xdot, np.float64)
        R = np.empty(self.N)
        a = np.empty(self.msr_len) if jacobian else None
        _lib.check(self._L.gb_matrix_fill_full_transient(self.h, _dp(x), _dp(xdot),
                                                         float(delta_t), float(theta), _dp(R),
                                                         _dp(a) if a is not None else None))
        return R, a

    def solve_transient_step(self, x, xdot, delta_t, theta, **opts):
        """One time step's Newton solve from the predicted (x, xdot):
        (x, xdot, converged, stats dict)."""
        x = np.ascontiguousarray(x, np.float64).copy()
        xdot = np.ascontiguousarray(xdot, np.float64).copy()
        o = self.newton_opts(**opts)
        conv = ctypes.c_int()
        st = _lib.NewtonStats()
        _lib.check(self._L.gb_solve_nonlinear_problem_transient(
            self.h, _dp(x), _dp(xdot), float(delta_t), float(theta), ctypes.byref(o),
            ctypes.byref(conv), ctypes.byref(st)))
        return x, xdot, bool(conv.value), _stats_dict(st)

    def solve_transient(self, num_steps, delta_t, theta=0.5, x0=None, **opts):
        """The reference's fixed-step time loop (gb_solve_transient) from x0
        (Dirichlet values applied if None): backward Euler for three steps,
        then theta.  Returns (solutions of every step [num_steps, N], stats
        dict with the per-step converged norms)."""
        x = self.dirichlet_init(np.zeros(self.N)) if x0 is None else np.ascontiguousarray(
            x0, np.float64).copy()
        xs = np.empty((num_steps, self.N))
        o = self.newton_opts(**opts)
        st = _lib.NewtonStats()
        done = ctypes.c_int()
        _lib.check(self._L.gb_solve_transient(self.h, _dp(x), int(num_steps), float(delta_t),
                                              float(theta), ctypes.byref(o), _dp(xs),
                                              ctypes.byref(st), ctypes.byref(done)))
        d = _stats_dict(st)
        d["steps_done"] = done.value
        d["step_residual_l2"] = [st.residual_l2[k] for k in range(min(num_steps, 64))]
        return xs, d

    def matrix_fill_full_device(self, d_x, d_R, d_vals, stream=None):
        """Device pointers; enqueued on ``stream`` (default: library stream)."""
        _lib.check(self._L.gb_matrix_fill_full_device(self.h, d_x, d_R, d_vals, stream))

    def status(self):
        _lib.check(self._L.gb_status(self.h))

    def set_material(self, material):
        """update_parameterC analogue: new material, same mesh and pattern."""
        from .problem import make_desc
        self.problem.material = material
        desc, keep = make_desc(self.problem)
        _lib.check(self._L.gb_set_material(self.h, ctypes.byref(desc.mat)))
        del keep

    def set_assembly_path(self, path):
        """Element kernel (gb_set_assembly_path): 0 automatic, 1 scalar FP64,
        2 / 3 FP64 DMMA variants, 4 sum factorisation (3-D Newtonian)."""
        _lib.check(self._L.gb_set_assembly_path(self.h, int(path)))

    def set_triangular_solve(self, mode):
        """ILU(0) solves: 0 sync-free sweeps, 1 level-scheduled graph,
        2 automatic (the default)."""
        _lib.check(self._L.gb_set_triangular_solve(self.h, int(mode)))

    def set_sweep_fault(self, spin_limit=0, reverse_lower=False):
        """Host-injected fault of the sync-free ILU(0) sweeps
        (gb_set_sweep_fault): polls per wait before it gives up (0: the
        default) and a reversed lower-sweep order on one CTA, whose waits can
        only end by giving up.  set_sweep_fault() restores the normal sweeps."""
        _lib.check(self._L.gb_set_sweep_fault(self.h, int(spin_limit), 1 if reverse_lower else 0))

    def scale_device(self, d_vals, d_R, d_scale=None):
        """row_sum_scaling_scale on device arrays (in place)."""
        _lib.check(self._L.gb_row_sum_scale_device(self.h, d_vals, d_R, d_scale))

    def linear_solve_device(self, d_vals, d_rhs, d_dx, **opts):
        o = self.newton_opts(**opts)
        its = ctypes.c_int()
        rr = ctypes.c_double()
        _lib.check(self._L.gb_linear_solve_device(self.h, d_vals, d_rhs, d_dx, ctypes.byref(o),
                                                  ctypes.byref(its), ctypes.byref(rr)))
        return its.value, rr.value

    # --- solve_nonlinear_problem
    def write_exodus(self, path, solutions, times=None, title="goma_gb300 solution"):
        """Exodus II results file of host solution vectors of this problem
        (the reference's variable names; goma_gb300.exodus)."""
        from .exodus import write_exodus
        write_exodus(path, self.problem, solutions, times, title)

    def newton_opts(self, **kw):
        """gb_newton_opts with the defaults of gb_newton_opts_default and the
        given fields (fp32_inner=True sets linear_precision to FP32 inner
        GMRES inside FP64 refinement, fp32_preconditioner=True to FP64
        flexible GMRES with the ILU(0) factorised and applied in FP32); an
        unknown name is an error rather than a silently ignored attribute."""
        o = _lib.NewtonOpts()
        self._L.gb_newton_opts_default(ctypes.byref(o))
        fields = {f[0] for f in o._fields_}
        for k, v in kw.items():
            if k in ("fp32_inner", "fp32_preconditioner"):
                mode = 1 if k == "fp32_inner" else 2
                if v:
                    o.linear_precision = mode
                elif o.linear_precision == mode:
                    o.linear_precision = 0
            elif k in fields:
                setattr(o, k, v)
            else:
                raise TypeError("unknown Newton option %r" % k)
        return o

    def solve_nonlinear_problem(self, x0=None, **opts):
        """Newton from x0 (host; Dirichlet values applied if x0 is None) to
        the scaled-residual tolerance.  Returns (x, converged, stats dict)."""
        x = self.dirichlet_init(np.zeros(self.N)) if x0 is None else np.ascontiguousarray(
            x0, np.float64).copy()
        o = self.newton_opts(**opts)
        conv = ctypes.c_int()
        st = _lib.NewtonStats()
        _lib.check(self._L.gb_solve_nonlinear_problem(self.h, _dp(x), ctypes.byref(o),
                                                      ctypes.byref(conv), ctypes.byref(st)))
        return x, bool(conv.value), _stats_dict(st)

    def solve_nonlinear_problem_device(self, d_x, **opts):
        o = self.newton_opts(**opts)
        conv = ctypes.c_int()
        st = _lib.NewtonStats()
        _lib.check(self._L.gb_solve_nonlinear_problem_device(self.h, d_x, ctypes.byref(o),
                                                             ctypes.byref(conv),
                                                             ctypes.byref(st)))
        return bool(conv.value), _stats_dict(st)

    def linear_solve(self, a_msr, rhs, **opts):
        """Host MSR (row-scaled) matrix and right-hand side -> dx."""
        a_msr = np.ascontiguousarray(a_msr, np.float64)
        rhs = np.ascontiguousarray(rhs, np.float64)
        dx = np.empty(self.N)
        o = self.newton_opts(**opts)
        its = ctypes.c_int()
        rr = ctypes.c_double()
        _lib.check(self._L.gb_linear_solve(self.h, _dp(a_msr), _dp(rhs), _dp(dx), ctypes.byref(o),
                                           ctypes.byref(its), ctypes.byref(rr)))
        return dx, its.value, rr.value

    def ilu0_factors(self, a_msr, fp32=False):
        """ILU(0) factors the linear solve would use for this row-scaled MSR
        matrix, returned in MSR layout (diagonal = U's, off-diagonal L and U)."""
        a_msr = np.ascontiguousarray(a_msr, np.float64)
        lu = np.empty(self.nnz)
        _lib.check(self._L.gb_ilu0_factors(self.h, _dp(a_msr), 1 if fp32 else 0, _dp(lu)))
        rowptr, colidx = self.csr_pattern()
        rows = np.repeat(np.arange(self.N), np.diff(rowptr))
        diag = colidx == rows
        out = np.empty(self.msr_len)
        out[:self.N] = lu[diag]
        out[self.N] = 0.0
        out[self.N + 1:] = lu[~diag]
        return out

    def csr_to_msr(self, d_vals):
        a = np.empty(self.msr_len)
        _lib.check(self._L.gb_csr_to_msr_host(self.h, d_vals, _dp(a)))
        return a


def _stats_dict(st):
    n = st.newton_its
    return {"newton_its": n, "linear_its": st.linear_its, "refinements": st.refinements,
            "residual_l2": [st.residual_l2[i] for i in range(min(n + 1, 64))],
            "residual_l1": [st.residual_l1[i] for i in range(min(n + 1, 64))],
            "residual_loo_steps": [st.residual_loo_steps[i] for i in range(min(n + 1, 64))],
            "residual_loo": st.residual_loo, "assemble_ms": st.assemble_ms,
            "scale_ms": st.scale_ms, "factor_ms": st.factor_ms, "solve_ms": st.solve_ms,
            "total_ms": st.total_ms, "factorizations": st.factorizations}
