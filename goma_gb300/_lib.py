"""ctypes loader of libgbnewton.so (the C ABI in include/gb_newton.h).

The product path goes through this library only: if it is missing or fails
to load, every call raises -- there is no CPU fallback.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgbnewton.so")

_lib = None


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
