"""ctypes binding of libimps_gb300.so (the C ABI declared in include/imps_gb300.h).

The library is built in-tree by ``imps_cpp_tools_gb300.build``.  There is no fallback: if the
library cannot be loaded every entry point raises ``ImpsError``.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

from . import build as _build

c_int, c_i64, c_dbl, c_vp = C.c_int, C.c_int64, C.c_double, C.c_void_p
P_i32 = C.POINTER(C.c_int32)
P_i64 = C.POINTER(C.c_int64)
# imps_apply_fn: int (*)(void* user, const double* in, double* out)
APPLY_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_void_p, C.c_void_p)
P_dbl = C.POINTER(C.c_double)
P_int = C.POINTER(C.c_int)

STATUS = {0: "ok", 1: "not converged", -1: "bad argument", -2: "inconsistent sector table",
          -3: "CUDA error", -4: "NaN/Inf detected", -5: "timeout", -6: "no CUDA device",
          -7: "out of device memory", -8: "unsupported",
          -9: "problem exceeds the fixed scratch of the no-allocation entry point"}

MEM_HOST, MEM_DEVICE = 0, 1
WHICH = {"LM": 0, "LR": 1, "SR": 2}
DIR_LEFT, DIR_RIGHT = 0, 1
PREC_FP64, PREC_BF16X6 = 0, 1


class ImpsError(RuntimeError):
    def __init__(self, status, where=""):
        super().__init__(f"{where}: imps status {status} ({STATUS.get(status, 'unknown')})")
        self.status = status


_PROTOS = {
    "imps_status_string": (C.c_char_p, [c_int]),
    "imps_version": (c_int, []),
    "imps_launch_count": (c_i64, []),
    "imps_ctx_create": (c_int, [c_int, C.POINTER(c_vp)]),
    "imps_ctx_destroy": (c_int, [c_vp]),
    "imps_ctx_set_stream": (c_int, [c_vp, c_vp]),
    "imps_ctx_synchronize": (c_int, [c_vp]),
    "imps_ctx_use_own_stream": (c_int, [c_vp]),
    "imps_layout_create": (c_int, [c_int, c_int, P_i32, P_i32, P_i32, P_i32, P_i32, C.POINTER(c_vp)]),
    "imps_layout_destroy": (c_int, [c_vp]),
    "imps_layout_nelem": (c_i64, [c_vp]),
    "imps_layout_nblocks": (c_int, [c_vp]),
    "imps_layout_nsym": (c_int, [c_vp]),
    "imps_layout_get": (c_int, [c_vp, P_i32, P_i32, P_i32, P_i32, P_i32, P_i64]),
    "imps_layout_bond": (c_int, [c_vp, c_int, C.POINTER(c_vp)]),
    "imps_plan_hac": (c_int, [c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_int, C.POINTER(c_vp)]),
    "imps_plan_hc": (c_int, [c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_int, c_int, P_i32, P_i32, P_dbl,
                             C.POINTER(c_vp)]),
    "imps_plan_tm": (c_int, [c_vp, c_int, C.POINTER(c_vp), c_int, c_vp, c_vp, C.POINTER(c_vp)]),
    "imps_plan_redop": (c_int, [c_vp, c_vp, c_int, c_int, P_i32, P_i32, P_dbl, c_int, C.POINTER(c_vp)]),
    "imps_plan_optm": (c_int, [c_vp, c_vp, c_vp, c_int, c_int, P_i32, P_i32, P_dbl, c_int, c_vp,
                               C.POINTER(c_vp)]),
    "imps_plan_mps_bd": (c_int, [c_vp, c_vp, c_vp, c_int, c_dbl, C.POINTER(c_vp)]),
    "imps_plan_grad_right": (c_int, [c_vp, c_vp, c_vp, C.POINTER(c_vp)]),
    "imps_plan_destroy": (c_int, [c_vp]),
    "imps_plan_derived_layout": (c_int, [c_vp, c_int, C.POINTER(c_vp)]),
    "imps_plan_info": (c_int, [c_vp, P_i64, P_i64, P_i64, P_int, P_int]),
    "imps_plan_slot_info": (c_int, [c_vp, c_int, P_int, P_i64]),
    "imps_plan_bind": (c_int, [c_vp, c_int, c_vp]),
    "imps_plan_prepare": (c_int, [c_vp]),
    "imps_plan_run": (c_int, [c_vp]),
    "imps_plan_table": (c_int, [c_vp, c_int, c_int, P_i64, P_i64, P_i32, P_i32, P_i32, P_i32, P_i64,
                                P_i32, P_i64, P_i32, P_dbl]),
    "imps_plan_set_precision": (c_int, [c_vp, c_int]),
    "imps_plan_autotune": (c_int, [c_vp, c_int, C.POINTER(c_int)]),
    "imps_plan_stage_shape": (c_int, [c_vp, c_int, C.POINTER(c_int), C.POINTER(c_int), C.POINTER(C.c_uint64)]),
    "imps_autotune_clear": (c_int, []),
    "imps_plan_replicate": (c_int, [c_vp, c_int, C.POINTER(c_vp)]),
    "imps_invert_e_fac_batch": (c_int, [c_vp, c_int, C.POINTER(c_vp), C.POINTER(c_vp), C.POINTER(c_dbl),
                                        C.POINTER(c_dbl), C.POINTER(c_vp), C.POINTER(c_vp), c_dbl, c_int, c_int,
                                        C.POINTER(c_int), C.POINTER(c_dbl)]),
    "imps_eigs_rs_batch_op": (c_int, [c_vp, c_int, c_i64, APPLY_FN, c_vp, c_vp, c_int, c_dbl, c_int, c_int,
                                      C.POINTER(c_dbl), C.POINTER(c_int), C.POINTER(c_int)]),
    "imps_hac_apply": (c_int, [c_vp, c_vp, c_vp, c_int]),
    "imps_hc_apply": (c_int, [c_vp, c_vp, c_vp, c_int]),
    "imps_tm_apply": (c_int, [c_vp, c_vp, c_vp, c_int]),
    "imps_tm_proj_apply": (c_int, [c_vp, c_vp, c_vp, c_vp, c_vp, c_int]),
    "imps_tm_apply_noalloc": (c_int, [c_vp, c_vp, c_vp, c_int, c_vp, c_vp, c_vp, c_vp]),
    "imps_eigs_rs": (c_int, [c_vp, c_vp, c_int, c_dbl, c_int, c_int, P_dbl, P_int]),
    "imps_invert_e_proj": (c_int, [c_vp, c_vp, c_vp, c_vp, c_int, c_vp, c_int, c_dbl, c_int, c_int,
                                   P_int, P_dbl]),
    "imps_tm_dominant": (c_int, [c_vp, c_vp, c_vp, c_int, c_dbl, c_int, P_dbl, P_int]),
    "imps_eigs_rs_op": (c_int, [c_vp, c_i64, APPLY_FN, c_vp, c_vp, c_int, c_int, c_dbl, c_int, c_int, P_dbl,
                                c_vp, P_int]),
    "imps_sector_svd_batch": (c_int, [c_int, C.POINTER(c_vp), C.POINTER(c_vp), C.POINTER(c_vp), C.POINTER(c_vp),
                                      C.POINTER(c_vp), c_int]),
    "imps_eigs_n": (c_int, [c_vp, c_vp, c_int, c_int, c_int, c_dbl, c_int, c_int, P_dbl, c_vp, c_vp, P_int]),
    "imps_eigs_n_op": (c_int, [c_vp, c_i64, APPLY_FN, c_vp, c_vp, c_int, c_int, c_int, c_dbl, c_int, c_int,
                               P_dbl, c_vp, c_vp, P_int]),
    "imps_plan_program": (c_int, [c_vp, c_int, P_i64, c_int, P_i32, P_i64, P_i64, P_dbl, C.POINTER(c_vp)]),
    "imps_plan_tm_mixed": (c_int, [c_vp, c_int, C.POINTER(c_vp), C.POINTER(c_vp), c_int, c_vp, c_vp,
                                   C.POINTER(c_vp)]),
    "imps_invert_e_fac": (c_int, [c_vp, c_vp, c_vp, c_dbl, c_dbl, c_vp, c_vp, c_int, c_dbl, c_int, c_int,
                                  P_int, P_dbl]),
    "imps_invert_e_proj_fac": (c_int, [c_vp, c_vp, c_vp, c_vp, c_vp, c_int, c_dbl, c_dbl, c_vp, c_vp, c_int,
                                       c_dbl, c_int, c_int, P_int, P_dbl]),
    "imps_grad_norm_right": (c_int, [c_vp, P_dbl]),
    "imps_dot": (c_int, [c_vp, c_vp, c_vp, c_i64, P_dbl]),
    "imps_plan_decomp": (c_int, [c_vp, c_vp, c_int, C.POINTER(c_vp)]),
    "imps_sector_qr": (c_int, [c_vp, c_vp, c_vp, c_vp, c_int]),
    "imps_sector_svd": (c_int, [c_vp, c_vp, c_vp, c_vp, c_vp, c_int]),
    "imps_sector_nullspace": (c_int, [c_vp, c_vp, c_vp, c_int]),
    "imps_sector_colscale": (c_int, [c_vp, c_vp, c_vp, c_dbl, c_int]),
    "imps_bd_trace_prod": (c_int, [c_vp, c_vp, c_vp, c_vp, P_dbl]),
    "imps_absmax": (c_int, [c_vp, c_vp, c_i64, P_dbl]),
    "imps_axpby": (c_int, [c_vp, c_dbl, c_vp, c_dbl, c_vp, c_i64]),
    "imps_sign_normalize": (c_int, [c_vp, c_vp, c_i64]),
}

_lib = None
_lock = threading.Lock()


def lib_path():
    return str(_build.LIB)


def load(build_if_needed: bool = True):
    """Load (building first if needed) the native library; raises if it is unavailable."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB
        if build_if_needed and (not path.exists() or _build._stale()):
            _build.build()
        if not path.exists():
            raise ImpsError(-8, f"native library missing at {path}")
        lib = C.CDLL(str(path), mode=os.RTLD_GLOBAL if hasattr(os, "RTLD_GLOBAL") else 0)
        for name, (res, args) in _PROTOS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def call(name, *args):
    """Call an entry point; raise ImpsError on a negative status, return the status otherwise."""
    st = getattr(load(), name)(*args)
    if isinstance(st, int) and st < 0:
        raise ImpsError(st, name)
    return st


def header_symbols():
    """Names of all functions declared in include/imps_gb300.h."""
    import re
    hdr = _build.INCLUDE / "imps_gb300.h"
    txt = hdr.read_text()
    return sorted(set(re.findall(r"\b(imps_[a-z0-9_]+)\s*\(", txt)))
