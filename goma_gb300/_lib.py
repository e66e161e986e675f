"""ctypes loader of libgbnewton.so (the C ABI in include/gb_newton.h).

The product path goes through this library only: if it is missing or fails
to load, every call raises -- there is no CPU fallback.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgbnewton.so")

_lib = None


class NewtonOpts(ctypes.Structure):
    """gb_newton_opts (include/gb_newton.h)."""
    _fields_ = [("max_newton", ctypes.c_int), ("residual_tol", ctypes.c_double),
                ("damping", ctypes.c_double), ("krylov_dim", ctypes.c_int),
                ("max_linear_its", ctypes.c_int), ("linear_tol", ctypes.c_double),
                ("linear_precision", ctypes.c_int), ("inner_tol", ctypes.c_double),
                ("max_refinements", ctypes.c_int), ("verbose", ctypes.c_int),
                ("forcing", ctypes.c_int), ("forcing_max", ctypes.c_double),
                ("factorization_reuse", ctypes.c_int)]


class NewtonStats(ctypes.Structure):
    """gb_newton_stats (include/gb_newton.h)."""
    _fields_ = [("newton_its", ctypes.c_int), ("linear_its", ctypes.c_int),
                ("refinements", ctypes.c_int), ("residual_l2", ctypes.c_double * 64),
                ("residual_loo", ctypes.c_double), ("assemble_ms", ctypes.c_double),
                ("scale_ms", ctypes.c_double), ("factor_ms", ctypes.c_double),
                ("solve_ms", ctypes.c_double), ("total_ms", ctypes.c_double),
                ("factorizations", ctypes.c_int), ("residual_l1", ctypes.c_double * 64),
                ("residual_loo_steps", ctypes.c_double * 64)]


MLP_NOALLOC_MAX_ACT = 1 << 20  # GB_MLP_NOALLOC_MAX_ACT of include/gb_newton.h


class GbError(RuntimeError):
    pass


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise GbError("libgbnewton.so is not built (run __graft_entry__.build() or "
                      "python goma_gb300/build.py)")
    L = ctypes.CDLL(LIB_PATH)
    vp, ip, dp = ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double)
    llp = ctypes.POINTER(ctypes.c_longlong)
    fp = ctypes.POINTER(ctypes.c_float)
    sig = {
        "gb_create": (ctypes.c_int, [vp, ctypes.POINTER(vp)]),
        "gb_destroy": (None, [vp]),
        "gb_last_error": (ctypes.c_char_p, []),
        "gb_num_unknowns": (ctypes.c_int, [vp]),
        "gb_msr_length": (ctypes.c_longlong, [vp]),
        "gb_csr_nnz": (ctypes.c_longlong, [vp]),
        "gb_num_colors": (ctypes.c_int, [vp]),
        "gb_msr_pattern": (ctypes.c_int, [vp, ip]),
        "gb_msr_pattern_host": (ctypes.c_int, [vp, ip, llp]),
        "gb_csr_pattern": (ctypes.c_int, [vp, llp, ip]),
        "gb_sweep_order_host": (ctypes.c_int, [vp, ctypes.c_int, ctypes.POINTER(ctypes.c_ushort),
                                               ip, ip]),
        "gb_csr_row": (ctypes.c_longlong, [vp, vp, ctypes.c_int, llp, ip, dp, ctypes.c_longlong]),
        "gb_matrix_fill_full_transient": (ctypes.c_int, [vp, dp, dp, ctypes.c_double,
                                                         ctypes.c_double, dp, dp]),
        "gb_matrix_fill_full_transient_device": (ctypes.c_int, [vp, vp, vp, ctypes.c_double,
                                                                ctypes.c_double, vp, vp, vp]),
        "gb_solve_nonlinear_problem_transient": (ctypes.c_int, [vp, dp, dp, ctypes.c_double,
                                                                ctypes.c_double,
                                                                ctypes.POINTER(NewtonOpts), ip,
                                                                ctypes.POINTER(NewtonStats)]),
        "gb_solve_transient": (ctypes.c_int, [vp, dp, ctypes.c_int, ctypes.c_double,
                                              ctypes.c_double, ctypes.POINTER(NewtonOpts), dp,
                                              ctypes.POINTER(NewtonStats), ip]),
        "gb_first_unknown": (ctypes.c_int, [vp, ip]),
        "gb_dirichlet_init": (ctypes.c_int, [vp, dp]),
        "gb_matrix_fill_full": (ctypes.c_int, [vp, dp, dp, dp]),
        "gb_matrix_fill_full_device": (ctypes.c_int, [vp, vp, vp, vp, vp]),
        "gb_status": (ctypes.c_int, [vp]),
        "gb_device_buffers": (ctypes.c_int, [vp, ctypes.POINTER(vp), ctypes.POINTER(vp),
                                             ctypes.POINTER(vp), ctypes.POINTER(vp),
                                             ctypes.POINTER(vp)]),
        "gb_stream": (vp, [vp]),
        "gb_csr_to_msr_host": (ctypes.c_int, [vp, vp, dp]),
        "gb_newton_opts_default": (None, [ctypes.POINTER(NewtonOpts)]),
        "gb_abi_struct_size": (ctypes.c_longlong, [ctypes.c_int]),
        "gb_solve_nonlinear_problem": (ctypes.c_int, [vp, dp, ctypes.POINTER(NewtonOpts), ip,
                                                      ctypes.POINTER(NewtonStats)]),
        "gb_solve_nonlinear_problem_device": (ctypes.c_int, [vp, vp, ctypes.POINTER(NewtonOpts),
                                                             ip, ctypes.POINTER(NewtonStats)]),
        "gb_row_sum_scale_device": (ctypes.c_int, [vp, vp, vp, vp]),
        "gb_linear_solve_device": (ctypes.c_int, [vp, vp, vp, vp, ctypes.POINTER(NewtonOpts), ip,
                                                  dp]),
        "gb_probe_fp64_peaks": (ctypes.c_int, [dp, dp]),
        "gb_probe_dmma_varying": (ctypes.c_int, [dp]),
        "gb_mlp_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                         ctypes.c_ulonglong, ctypes.POINTER(vp)]),
        "gb_mlp_destroy": (None, [vp]),
        "gb_mlp_num_params": (ctypes.c_int, [vp]),
        "gb_mlp_get_params": (ctypes.c_int, [vp, fp]),
        "gb_mlp_set_params": (ctypes.c_int, [vp, fp]),
        "gb_mlp_get_grads": (ctypes.c_int, [vp, fp]),
        "gb_mlp_forward_device": (ctypes.c_int, [vp, vp, ctypes.c_int, vp]),
        "gb_mlp_forward_noalloc": (ctypes.c_int, [vp, vp, ctypes.c_int, vp, vp]),
        "gb_mlp_loss_grad_device": (ctypes.c_int, [vp, vp, vp, vp, ctypes.c_int, fp]),
        "gb_mlp_adam_step": (ctypes.c_int, [vp, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                            ctypes.c_float]),
        "gb_mlp_train_device": (ctypes.c_int, [vp, vp, vp, vp, ctypes.c_int, ctypes.c_int,
                                               ctypes.c_int, ctypes.c_float, ctypes.c_ulonglong,
                                               fp]),
        "gb_set_material": (ctypes.c_int, [vp, vp]),
        "gb_set_assembly_path": (ctypes.c_int, [vp, ctypes.c_int]),
        "gb_set_element_density": (ctypes.c_int, [vp, dp]),
        "gb_set_ilu_ordering": (ctypes.c_int, [vp, ctypes.c_int]),
        "gb_ilu_permutation_host": (ctypes.c_int, [vp, ip, ip, ip, ctypes.POINTER(ctypes.c_longlong),
                                                   ip, ctypes.POINTER(ctypes.c_longlong)]),
        "gb_set_triangular_solve": (ctypes.c_int, [vp, ctypes.c_int]),
        "gb_set_sweep_fault": (ctypes.c_int, [vp, ctypes.c_longlong, ctypes.c_int]),
        "gb_ilu0_factors": (ctypes.c_int, [vp, dp, ctypes.c_int, dp]),
        "gb_kernel_timing": (ctypes.c_int, [vp, ctypes.c_int, dp, llp]),
        "gb_linear_solve": (ctypes.c_int, [vp, dp, dp, dp, ctypes.POINTER(NewtonOpts), ip, dp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def check(rc):
    if rc != 0:
        raise GbError(load().gb_last_error().decode())
    return rc
