"""ctypes binding of liblexgb.so (the C ABI declared in include/lexgb.h).

The library is built in-tree by ``lex_gb300.build``; importing this module never falls
back to anything else: a missing or unloadable library raises immediately.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liblexgb.so")

LEXGB_OK, LEXGB_ERR_ARG, LEXGB_ERR_CUDA, LEXGB_ERR_NAN, LEXGB_ERR_TIMEOUT, LEXGB_ERR_STATE, LEXGB_ERR_ALLOC = range(7)
LEXGB_F32, LEXGB_F64 = 0, 1

DIAGNOSTICS = ["mass_div", "adv_theta", "adv_qv", "adv_u", "adv_v", "adv_w", "buoy_w", "theta_rho",
               "pgf_u", "pgf_v", "pgf_w", "adv_pi", "sgs_u", "sgs_v", "sgs_w", "sgs_theta", "sgs_qv",
               "n2", "km"]

KERNELS = ["acoustic", "div_trho", "adv_scalars", "adv_momentum", "smag_a", "smag_b", "acoustic_pair",
           "acoustic_stage"]

# every entry point include/lexgb.h declares: name -> (restype, argtypes)
_P = ctypes.c_void_p
_I = ctypes.c_int
_D = ctypes.POINTER(ctypes.c_double)


class Config(ctypes.Structure):
    """Mirror of ``lexgb_config``."""
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
                ("dx", ctypes.c_double), ("dy", ctypes.c_double), ("dz", ctypes.c_double),
                ("dt", ctypes.c_double), ("n_sound", ctypes.c_int), ("turb_opt", ctypes.c_int),
                ("cor_opt", ctypes.c_int), ("f_cor", ctypes.c_double), ("theta_ref", ctypes.c_double),
                ("acoustic_pairs", ctypes.c_int), ("l2_persist", ctypes.c_int), ("cs", ctypes.c_double),
                ("acoustic_kernel", ctypes.c_int)]

ACOUSTIC_KERNELS = {"auto": 0, "rows": 1, "tile": 2, "persistent": 3}


SIGNATURES = {
    "lexgb_default_config": (_I, [ctypes.POINTER(Config)]),
    "lexgb_create": (_I, [ctypes.POINTER(Config), ctypes.POINTER(_P)]),
    "lexgb_destroy": (_I, [_P]),
    "lexgb_set_stream": (_I, [_P, _P]),
    "lexgb_set_base_columns": (_I, [_P, _D, _D, _D, _D]),
    "lexgb_integrate_base_state": (_I, [_P, _D, _D, _D, _D]),
    "lexgb_upload_state": (_I, [_P, ctypes.POINTER(_P), _I]),
    "lexgb_download_state": (_I, [_P, ctypes.POINTER(_P), _I]),
    "lexgb_step": (_I, [_P, _I, _I]),
    "lexgb_step_record": (_I, [_P]),
    "lexgb_download_stage": (_I, [_P, _I, ctypes.POINTER(_P), ctypes.POINTER(_P)]),
    "lexgb_diagnose": (_I, [_P, _I, _D]),
    "lexgb_budget": (_I, [_P, _D, _I]),
    "lexgb_check_finite": (_I, [_P, ctypes.POINTER(ctypes.c_longlong)]),
    "lexgb_synchronize": (_I, [_P]),
    "lexgb_set_barrier_limit": (_I, [_P, ctypes.c_longlong]),
    "lexgb_acoustic_kernel": (_I, [_P, ctypes.POINTER(ctypes.c_int)]),
    "lexgb_state_device_ptrs": (_I, [_P, ctypes.POINTER(_P)]),
    "lexgb_step_kernel_count": (_I, [_P, ctypes.POINTER(ctypes.c_int)]),
    "lexgb_time_kernel": (_I, [_P, _I, _I, ctypes.POINTER(ctypes.c_float)]),
    "lexgb_budget_noalloc": (_I, [_I, _I, _I, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                  ctypes.POINTER(_P), _P, _P, _P, _P]),
    "lexgb_set_state_interior": (_I, [_P, ctypes.POINTER(_P), _I]),
    "lexgb_get_state_interior": (_I, [_P, ctypes.POINTER(_P), _I]),
    "lexgb_step_vjp": (_I, [_P, _I, ctypes.POINTER(_P), ctypes.POINTER(_P), _I]),
    "lexgb_step_keep": (_I, [_P]),
    "lexgb_step_vjp_kept": (_I, [_P, ctypes.POINTER(_P), ctypes.POINTER(_P), _I]),
    "lexgb_cnn_conv3d": (_I, [_I, _I, _I, _I, _I, _P, _P, _P, _P, _P, _P, _I, _I, _P]),
    "lexgb_cnn_gelu_bwd": (_I, [ctypes.c_longlong, _I, _I, _P, _P, _P, _P]),
    "lexgb_cnn_set_kernel": (_I, [_I]),
    "lexgb_cnn_take_timeouts": (_I, [_P]),
    "lexgb_cnn_conv3d_dw": (_I, [_I, _I, _I, _I, _I, _I, _P, _P, _P, _P, _P]),
    "lexgb_cnn_adam": (_I, [ctypes.c_longlong, _P, _P, _P, _P, _P, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                            ctypes.c_float, _I, _P]),
    "lexgb_set_sgs_net": (_I, [_P, ctypes.POINTER(_P), ctypes.POINTER(_P), _P, _P, _P, _I]),
    "lexgb_set_cs": (_I, [_P, ctypes.c_double]),
    "lexgb_get_cs_grad": (_I, [_P, ctypes.POINTER(ctypes.c_double), _I]),
    "lexgb_last_error": (_I, [ctypes.c_char_p, ctypes.c_size_t]),
}

_lib = None


class LexError(RuntimeError):
    """A non-zero status from the C ABI, with the library's message."""

    def __init__(self, code, msg):
        super().__init__("lexgb error %d: %s" % (code, msg))
        self.code = code


def load():
    """Load liblexgb.so and bind every entry point (raises if absent)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError("lex_gb300 native library not built: %s is missing "
                          "(run `python -m lex_gb300.build`)" % LIB_PATH)
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def last_error():
    lib = load()
    buf = ctypes.create_string_buffer(4096)
    lib.lexgb_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(status):
    if status != LEXGB_OK:
        raise LexError(status, last_error())
    return status
