"""ctypes binding of the CPU oracle (oracle/gb_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke``
and by the CPU-baseline leg of ``bench.py``, always as the checker or the
timed CPU reference, never as part of the product path.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liborc.so")
SRCS = [os.path.join(HERE, "gb_oracle.c"), os.path.join(HERE, "mesh_gen.c")]


def build(force=False):
    """Compile the oracle (plain C, portable flags) into oracle/liborc.so."""
    newest = max(os.path.getmtime(s) for s in SRCS + [os.path.join(HERE, "gb_oracle.h"),
                                                       os.path.join(HERE, "mesh_gen.h")])
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    tmp = LIB + ".tmp%d" % os.getpid()
    subprocess.run(["gcc", "-std=gnu11", "-O2", "-fPIC", "-shared", "-o", tmp] + SRCS + ["-lm"],
                   check=True)
    os.replace(tmp, LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        vp, ip, dp = ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double)
        L.orc_create.restype = vp
        L.orc_create.argtypes = [vp]
        L.orc_destroy.argtypes = [vp]
        L.orc_num_unknowns.argtypes = [vp]
        L.orc_msr_len.restype = ctypes.c_long
        L.orc_msr_len.argtypes = [vp]
        L.orc_msr_pattern.argtypes = [vp, ip]
        L.orc_first_unknown.argtypes = [vp, ip]
        L.orc_dirichlet_mask.argtypes = [vp, ip]
        L.orc_dirichlet_init.argtypes = [vp, dp]
        L.orc_matrix_fill.argtypes = [vp, dp, dp, dp, ctypes.c_int, ctypes.c_int]
        L.orc_matrix_fill_list.argtypes = [vp, dp, dp, dp, ip, ctypes.c_int]
        L.orc_element_colors.argtypes = [vp, ip]
        L.orc_element.argtypes = [vp, ctypes.c_int, dp, dp, dp, ctypes.c_int]
        L.orc_local_size.argtypes = [vp]
        L.orc_element_dofs.argtypes = [vp, ctypes.c_int, ip]
        L.orc_row_sum_scale.argtypes = [vp, dp, dp, dp]
        L.orc_newton.argtypes = [vp, dp, ctypes.c_int, ctypes.c_double, dp]
        L.orc_set_transient.argtypes = [vp, dp, ctypes.c_double]
        L.orc_newton_transient.argtypes = [vp, dp, dp, ctypes.c_double, ctypes.c_int,
                                           ctypes.c_double, dp]
        L.orc_ilu0.argtypes = [vp, dp, ctypes.c_double, dp]
        L.orc_gmres_ilu0.argtypes = [vp, dp, dp, dp, dp, ctypes.c_int, ctypes.c_int,
                                     ctypes.c_double, ip, dp]
        L.orc_newton_gmres.argtypes = [vp, dp, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                       ctypes.c_int, ctypes.c_int, ctypes.c_double, ip, dp]
        L.orc_mesh_sizes.argtypes = [ctypes.c_char_p, ip, ip, ip]
        L.orc_mesh_fill.argtypes = [ctypes.c_char_p, dp, ip, ip, ip]
        _lib = L
    return _lib


def _p(a, t):
    return a.ctypes.data_as(ctypes.POINTER(t))


class Oracle:
    """CPU restatement of the reference path for one problem."""

    def __init__(self, problem):
        from goma_gb300.problem import make_desc
        self._desc, self._keep = make_desc(problem)
        self.h = lib().orc_create(ctypes.byref(self._desc))
        if not self.h:
            raise RuntimeError("orc_create failed")
        self.N = lib().orc_num_unknowns(self.h)
        self.msr_len = lib().orc_msr_len(self.h)
        self.nloc = lib().orc_local_size(self.h)
        self.num_elems = problem.mesh.num_elems

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None

    def ija(self):
        out = np.empty(self.msr_len, np.int32)
        lib().orc_msr_pattern(self.h, _p(out, ctypes.c_int))
        return out

    def first_unknown(self, num_nodes):
        out = np.empty(num_nodes + 1, np.int32)
        lib().orc_first_unknown(self.h, _p(out, ctypes.c_int))
        return out

    def dirichlet_mask(self):
        out = np.empty(self.N, np.int32)
        lib().orc_dirichlet_mask(self.h, _p(out, ctypes.c_int))
        return out.astype(bool)

    def dirichlet_init(self, x):
        x = np.ascontiguousarray(x, np.float64).copy()
        lib().orc_dirichlet_init(self.h, _p(x, ctypes.c_double))
        return x

    def matrix_fill(self, x, jacobian=True, e0=0, e1=None, xdot=None, delta_t=None, theta=0.0):
        """Returns (R, a_msr or None, status).  With xdot (and delta_t,
        theta) the transient terms: mass terms of xdot, their sensitivity
        (1 + 2 theta) / delta_t."""
        x = np.ascontiguousarray(x, np.float64)
        R = np.zeros(self.N)
        a = np.zeros(self.msr_len) if jacobian else None
        if xdot is not None:
            xdot = np.ascontiguousarray(xdot, np.float64)
            lib().orc_set_transient(self.h, _p(xdot, ctypes.c_double),
                                    (1.0 + 2.0 * theta) / delta_t)
        try:
            st = lib().orc_matrix_fill(self.h, _p(x, ctypes.c_double), _p(R, ctypes.c_double),
                                       _p(a, ctypes.c_double) if a is not None else None, e0,
                                       self.num_elems if e1 is None else e1)
        finally:
            if xdot is not None:
                lib().orc_set_transient(self.h, None, 0.0)
        return R, a, st

    def newton_transient(self, x0, xdot0, delta_t, theta, max_it=40, tol=1e-10):
        """One time step's Newton solve from the predicted (x0, xdot0):
        (x, xdot, iterations or -1)."""
        x = np.ascontiguousarray(x0, np.float64).copy()
        xd = np.ascontiguousarray(xdot0, np.float64).copy()
        norms = np.full(max_it, np.nan)
        it = lib().orc_newton_transient(self.h, _p(x, ctypes.c_double), _p(xd, ctypes.c_double),
                                        (1.0 + 2.0 * theta) / delta_t, max_it, tol,
                                        _p(norms, ctypes.c_double))
        return x, xd, it

    def transient_run(self, x0, nsteps, delta_t, theta, tol=1e-10, max_it=40):
        """The reference's fixed-step transient loop (solve_problem,
        src/rf_solve.c:1138-2601, with a constant delta_t): histories start
        at x0 with zero time derivatives; the first three steps are backward
        Euler (theta = 0, :1378-1386), then the given theta; each step
        predicts x and xdot (predict_solution, :2767), solves, and shifts
        the histories (:2359-2366).  Returns the solution after every
        step."""
        x = self.dirichlet_init(x0)
        x_old = x.copy()
        x_older = x.copy()
        x_oldest = x.copy()
        xd_old = np.zeros_like(x)
        xd_older = np.zeros_like(x)
        out = []
        for nt in range(nsteps):
            th = 0.0 if nt < 3 else theta
            x, xd = predict(delta_t, delta_t, delta_t, th, x_old, x_older, x_oldest, xd_old,
                            xd_older)
            x, xd, it = self.newton_transient(x, xd, delta_t, th, max_it, tol)
            if it < 0:
                raise RuntimeError("oracle transient step %d did not converge" % nt)
            out.append(x.copy())
            xd_older, xd_old = xd_old, xd
            x_oldest, x_older, x_old = x_older, x_old, x
        return out


    def element(self, e, x, apply_bc=True):
        x = np.ascontiguousarray(x, np.float64)
        Re = np.zeros(self.nloc)
        Je = np.zeros((self.nloc, self.nloc))
        st = lib().orc_element(self.h, e, _p(x, ctypes.c_double), _p(Re, ctypes.c_double),
                               _p(Je, ctypes.c_double), 1 if apply_bc else 0)
        g = np.empty(self.nloc, np.int32)
        lib().orc_element_dofs(self.h, e, _p(g, ctypes.c_int))
        return Re, Je, g, st

    def ilu0(self, a, tau=1e-4):
        """ILU(0) factors of the MSR matrix a (same layout), pivot floor tau."""
        a = np.ascontiguousarray(a, np.float64)
        lu = np.empty(self.msr_len)
        if lib().orc_ilu0(self.h, _p(a, ctypes.c_double), tau, _p(lu, ctypes.c_double)) != 0:
            raise MemoryError("orc_ilu0")
        return lu

    def row_sum_scale(self, a, R):
        a = a.copy()
        R = R.copy()
        s = np.empty(self.N)
        lib().orc_row_sum_scale(self.h, _p(a, ctypes.c_double), _p(R, ctypes.c_double),
                                _p(s, ctypes.c_double))
        return a, R, s

    def newton(self, x0, max_it=40, tol=1e-10):
        x = np.ascontiguousarray(x0, np.float64).copy()
        norms = np.full(max_it, np.nan)
        it = lib().orc_newton(self.h, _p(x, ctypes.c_double), max_it, tol,
                              _p(norms, ctypes.c_double))
        return x, it, norms[:max(it + 1, 0)] if it >= 0 else norms

    def gmres_ilu0(self, a, lu, b, krylov=30, maxit=500, tol=1e-8):
        """ILU(0)-preconditioned GMRES(krylov) on the MSR system a x = b from
        x = 0: (x, converged, iterations, relative residual)."""
        a = np.ascontiguousarray(a, np.float64)
        lu = np.ascontiguousarray(lu, np.float64)
        b = np.ascontiguousarray(b, np.float64)
        x = np.empty(self.N)
        its = ctypes.c_int()
        rel = ctypes.c_double()
        st = lib().orc_gmres_ilu0(self.h, _p(a, ctypes.c_double), _p(lu, ctypes.c_double),
                                  _p(b, ctypes.c_double), _p(x, ctypes.c_double), krylov, maxit,
                                  tol, ctypes.byref(its), ctypes.byref(rel))
        if st < 0:
            raise MemoryError("orc_gmres_ilu0")
        return x, st == 0, its.value, rel.value

    def newton_gmres(self, x0, max_it=40, tol=1e-10, linear_tol=1e-8, krylov=30,
                     max_linear_its=4000, tau=1e-4):
        """Newton with ILU(0)-GMRES(krylov) linear solves (the reference's
        solver settings): (x, Newton iterations or -1, total Krylov
        iterations, scaled-residual L2 norms)."""
        x = np.ascontiguousarray(x0, np.float64).copy()
        norms = np.full(max_it, np.nan)
        lin = ctypes.c_int()
        it = lib().orc_newton_gmres(self.h, _p(x, ctypes.c_double), max_it, tol, linear_tol,
                                    krylov, max_linear_its, tau, ctypes.byref(lin),
                                    _p(norms, ctypes.c_double))
        return x, it, lin.value, norms[:max(it + 1, 0)] if it >= 0 else norms


class ParallelFill:
    """The oracle's matrix_fill_full over many host threads, for timing the
    reference's CPU assembly of a whole problem: per call, the caller's
    zeroing of R and of the MSR values (src/mm_sol_nonlinear.c:1114-1120),
    then the element loop (src/mm_fill.c:158-312) colour by colour.  Each
    colour's elements (no two share a node, so they touch disjoint rows) are
    split into `threads` chunks that add into one shared R and one shared
    MSR array; a colour starts when the previous one is done.  The sums of a
    row are taken in colour order rather than element order, so results
    match the serial fill to rounding, not bitwise."""

    def __init__(self, o, threads):
        import concurrent.futures
        self.o = o
        self.threads = max(1, int(threads))
        color = np.empty(o.num_elems, np.int32)
        nc = lib().orc_element_colors(o.h, _p(color, ctypes.c_int))
        if nc < 0:
            raise RuntimeError("orc_element_colors failed")
        self.num_colors = nc
        self.chunks = []
        for k in range(nc):
            els = np.flatnonzero(color == k).astype(np.int32)
            self.chunks.append([np.ascontiguousarray(c) for c in
                                np.array_split(els, self.threads) if len(c)])
        self.R = np.zeros(o.N)
        self.a = np.zeros(o.msr_len)
        self.pool = concurrent.futures.ThreadPoolExecutor(self.threads)

    def close(self):
        self.pool.shutdown()

    def _zero(self, arr):
        n = arr.size
        bounds = np.linspace(0, n, self.threads + 1).astype(np.int64)
        base = arr.ctypes.data

        def z(i):
            ctypes.memset(base + 8 * int(bounds[i]), 0, 8 * int(bounds[i + 1] - bounds[i]))

        list(self.pool.map(z, range(self.threads)))

    def __call__(self, x):
        """R and the MSR values of the state x (into self.R, self.a);
        returns 0, or -1 on a non-positive Jacobian determinant."""
        L = lib()
        x = np.ascontiguousarray(x, np.float64)
        self._zero(self.R)
        self._zero(self.a)
        xp, Rp, ap = (_p(v, ctypes.c_double) for v in (x, self.R, self.a))
        status = 0
        for col in self.chunks:
            sts = list(self.pool.map(
                lambda c: L.orc_matrix_fill_list(self.o.h, xp, Rp, ap, _p(c, ctypes.c_int),
                                                 len(c)), col))
            status = min([status] + sts)
        return status


def mesh_from_spec(spec):
    """The oracle generator's mesh: (coords, conn, [node sets])."""
    L = lib()
    nn, ne, st = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    if L.orc_mesh_sizes(spec.encode(), ctypes.byref(nn), ctypes.byref(ne), ctypes.byref(st)):
        raise ValueError(spec)
    dim = 3 if spec.startswith("hex27") else 2
    npe = 27 if dim == 3 else 9
    coords = np.empty((nn.value, dim))
    conn = np.empty((ne.value, npe), np.int32)
    lens = np.empty(6, np.int32)
    nodes = np.empty(max(st.value, 1), np.int32)
    L.orc_mesh_fill(spec.encode(), _p(coords, ctypes.c_double), _p(conn, ctypes.c_int),
                    _p(lens, ctypes.c_int), _p(nodes, ctypes.c_int))
    sets, off = [], 0
    for n in lens:
        sets.append(nodes[off:off + n].copy())
        off += n
    return coords, conn, sets


def predict(dt, dt_old, dt_older, theta, x_old, x_older, x_oldest, xd_old, xd_older):
    """predict_solution (src/rf_solve.c:2767-2834): the trapezoid rule's
    second-order extrapolation for theta = 0.5, else the first-order one;
    xdot consistent with the predicted x."""
    if theta == 0.5:
        c1 = dt * (dt + dt_old) / dt_older / (dt_older + dt_old)
        c2 = -dt * (dt + dt_old + dt_older) / (dt_old * dt_older)
        c3 = (dt + dt_old + dt_older) * (dt + dt_old) / dt_old / (dt_older + dt_old)
        x = c3 * x_old + c2 * x_older + c1 * x_oldest
    else:
        c1 = dt * (1.0 + theta * dt / dt_old)
        c2 = theta * dt * dt / dt_old
        x = x_old + c1 * xd_old - c2 * xd_older
    xd = (1.0 + 2.0 * theta) / dt * (x - x_old) - 2.0 * theta * xd_old
    return x, xd
