"""ctypes binding of the C ABI (include/imsrg_gb300.h).

Loads imsrg_gb300/_build/libimsrg_gb300.so, building it first if the sources
are newer.  There is no fallback: if the library cannot be built or loaded,
importing raises.
"""

import ctypes
import os
import threading

from . import build as _build

OK = 0
ERR_ARG = 1
ERR_CUDA = 2
ERR_UNSUPPORTED = 3
ERR_NOMEM = 4
ERR_KERNEL = 5
ERR_DIVERGED = 6
ERR_IO = 7
PREC_FP64 = 0
PREC_SPLIT = 1

_lock = threading.Lock()
_lib = None

P = ctypes.c_void_p
I = ctypes.c_int
IP = ctypes.POINTER(ctypes.c_int)
D = ctypes.c_double
DP = ctypes.POINTER(ctypes.c_double)
LL = ctypes.c_longlong
LLP = ctypes.POINTER(ctypes.c_longlong)

# name -> (restype, argtypes); every function declared in include/imsrg_gb300.h
SIGNATURES = {
    "imsrg_last_error": (ctypes.c_char_p, []),
    "imsrg_space_create": (I, [I, I, IP, IP, IP, IP, DP, ctypes.POINTER(P)]),
    "imsrg_space_create_reference": (I, [I, I, I, ctypes.POINTER(P)]),
    "imsrg_space_destroy": (None, [P]),
    "imsrg_space_sizes": (I, [P, IP, IP, LLP]),
    "imsrg_space_orbit": (I, [P, I, IP, IP, IP, IP, DP]),
    "imsrg_space_channel": (I, [P, I, IP, IP, IP, IP, LLP]),
    "imsrg_space_channel_kets": (I, [P, I, IP, IP]),
    "imsrg_space_cc_channel": (I, [P, I, IP, IP, IP, IP, IP, IP]),
    "imsrg_space_sixj": (I, [P, I, I, I, I, I, I, DP]),
    "imsrg_space_pandya_layout": (I, [P, I, IP, IP, LLP, LLP]),
    "imsrg_pandya_transform": (I, [P, I, P, P]),
    "imsrg_op_create": (I, [P, I, ctypes.POINTER(P)]),
    "imsrg_op_create_tensor": (I, [P, I, I, I, I, ctypes.POINTER(P)]),
    "imsrg_op_rank": (I, [P, IP, IP, IP, LLP]),
    "imsrg_space_tensor_layout": (I, [P, I, I, I, I, IP, IP, LLP, IP, LLP]),
    "imsrg_space_ninej": (I, [P, I, I, I, I, I, I, I, I, I, DP]),
    "imsrg_space_wait_selftest": (I, [P, ctypes.c_uint, ctypes.POINTER(ctypes.c_longlong),
                                      ctypes.POINTER(ctypes.c_uint), P]),
    "imsrg_commutator_scalar_tensor": (I, [P, P, P, I, P]),
    "imsrg_comm111st": (I, [P, P, P, P]),
    "imsrg_comm121st": (I, [P, P, P, P]),
    "imsrg_comm122st": (I, [P, P, P, P]),
    "imsrg_comm222_pp_hh_221st": (I, [P, P, P, I, P]),
    "imsrg_comm222_phst": (I, [P, P, P, I, P]),
    "imsrg_op_destroy": (None, [P]),
    "imsrg_op_hermiticity": (I, [P, IP]),
    "imsrg_op_set_hermiticity": (I, [P, I]),
    "imsrg_op_upload": (I, [P, DP, P]),
    "imsrg_op_download": (I, [P, DP, P]),
    "imsrg_op_device_arena": (I, [P, ctypes.POINTER(P)]),
    "imsrg_op_zero": (I, [P, P]),
    "imsrg_op_copy": (I, [P, P, P]),
    "imsrg_op_scale": (I, [P, D, P]),
    "imsrg_op_axpy": (I, [P, D, P, P]),
    "imsrg_op_norm": (I, [P, DP, P]),
    "imsrg_op_write_binary": (I, [P, ctypes.c_char_p, P]),
    "imsrg_op_read_binary": (I, [P, ctypes.c_char_p, P]),
    "imsrg_op_fill_random": (I, [P, ctypes.c_ulonglong, P]),
    "imsrg_comm110ss": (I, [P, P, P, P]),
    "imsrg_comm220ss": (I, [P, P, P, P]),
    "imsrg_comm111ss": (I, [P, P, P, P]),
    "imsrg_comm121ss": (I, [P, P, P, P]),
    "imsrg_comm122ss": (I, [P, P, P, P]),
    "imsrg_comm221ss": (I, [P, P, P, P]),
    "imsrg_comm122ss_noalloc": (I, [P, P, P, P, I, P]),
    "imsrg_comm222_pp_hhss": (I, [P, P, P, I, P]),
    "imsrg_comm222_pp_hh_221ss": (I, [P, P, P, I, P]),
    "imsrg_comm222_phss": (I, [P, P, P, I, P]),
    "imsrg_commutator_scalar_scalar": (I, [P, P, P, I, P]),
    "imsrg_set_term": (I, [ctypes.c_char_p, I]),
    "imsrg_get_term": (I, [ctypes.c_char_p, IP]),
    "imsrg_batch_create": (I, [I, ctypes.POINTER(P), ctypes.POINTER(P), ctypes.POINTER(P), I, ctypes.POINTER(P)]),
    "imsrg_batch_destroy": (None, [P]),
    "imsrg_batch_launch": (I, [P, P]),
    "imsrg_batch_sync": (I, [P, P]),
    "imsrg_batch_info": (I, [P, IP, IP, IP, LLP]),
    "imsrg_space_zbar_layout": (I, [P, I, IP, IP, LLP, LLP]),
    "imsrg_add_inverse_pandya": (I, [P, P, I, P]),
    "imsrg_space_set_tuning": (I, [P, ctypes.c_char_p, I]),
    "imsrg_space_get_tuning": (I, [P, ctypes.c_char_p, IP]),
    "imsrg_space_describe_tuning": (I, [P, ctypes.c_char_p, I]),
    "imsrg_space_defer_status": (I, [P, I]),
    "imsrg_space_check_status": (I, [P, P]),
    "imsrg_set_default_precision": (I, [I]),
    "imsrg_get_default_precision": (I, [IP]),
    "imsrg_bch_transform": (I, [P, P, P, D, I, IP, P]),
    "imsrg_bch_product": (I, [P, P, P, D, I, IP, P]),
    "imsrg_generator_update": (I, [P, P, I, I, D, D, I, P]),
    "imsrg_solver_create": (I, [P, ctypes.POINTER(P)]),
    "imsrg_solver_destroy": (None, [P]),
    "imsrg_solver_set": (I, [P, ctypes.c_char_p, D]),
    "imsrg_solver_get": (I, [P, ctypes.c_char_p, DP]),
    "imsrg_solver_set_generator": (I, [P, ctypes.c_char_p, P]),
    "imsrg_solver_set_scratch_dir": (I, [P, ctypes.c_char_p]),
    "imsrg_solver_set_denominator_partitioning": (I, [P, ctypes.c_char_p]),
    "imsrg_solver_solve": (I, [P, I, P]),
    "imsrg_solver_hs": (I, [P, ctypes.POINTER(P)]),
    "imsrg_solver_eta": (I, [P, ctypes.POINTER(P)]),
    "imsrg_solver_omega": (I, [P, I, ctypes.POINTER(P)]),
    "imsrg_solver_add_operator": (I, [P, P, IP, P]),
    "imsrg_solver_get_operator": (I, [P, I, ctypes.POINTER(P)]),
    "imsrg_solver_history": (I, [P, I, IP, DP, DP, DP, DP, IP]),
    "imsrg_solver_transform": (I, [P, P, P, I, P]),
    "imsrg_solver_inverse_transform": (I, [P, P, P, I, P]),
    "imsrg_profiler_enable": (I, [I]),
    "imsrg_profiler_reset": (I, []),
    "imsrg_profiler_get": (I, [ctypes.c_char_p, DP, LLP]),
    "imsrg_profiler_names": (I, [ctypes.c_char_p, I]),
    "imsrg_kernel_launches": (LL, []),
}


class IMSRGError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("imsrg_gb300 error %d: %s" % (code, msg))
        self.code = code


def lib():
    """The loaded library (built on first use)."""
    global _lib
    with _lock:
        if _lib is None:
            path = _build.build()
            L = ctypes.CDLL(path)
            for name, (res, args) in SIGNATURES.items():
                f = getattr(L, name)
                f.restype = res
                f.argtypes = args
            _lib = L
    return _lib


def library_path():
    return _build.LIB


def check(rc):
    if rc != OK:
        msg = lib().imsrg_last_error()
        raise IMSRGError(rc, msg.decode() if msg else "")
    return rc
