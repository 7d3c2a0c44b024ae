"""ctypes binding of libpoyalgn.so (the C ABI in include/poyalgn.h).

The library is the only compute path: importing this module on a machine
without the built library, or calling into it without a CUDA device, raises.
There is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
# POYALGN_LIBRARY selects another build of the library (same C ABI)
LIB_PATH = os.environ.get("POYALGN_LIBRARY") or os.path.join(HERE, "libpoyalgn.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "poyalgn.h")

_P = C.c_void_p
_I = C.c_int
_I64 = C.c_int64

# POYALGN_* return codes
EINVAL, ENOMEM, ECUDA, EUNSUPPORTED, EPAIR, EBUSY = -1, -2, -3, -4, -5, -6
PAIR_STATUS = {0: "ok", -2: "output capacity exceeded", -3: "median should not be 0",
               -4: "empty sequence or empty median", -5: "band wider than the largest pipeline",
               -6: "sequence too long", -7: "state outside the alphabet",
               -8: "band doubling did not stop", -9: "speculative pass not run",
               -11: "closest: a position with no state", -12: "rerun (arena full)",
               -13: "traceback leaves the band", 1: "not processed"}


class PoyAlgnError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"poyalgn error {code}: {msg}")
        self.code = code


_SIGS = {
    "poyalgn_init": (_I, [_I, C.POINTER(_P)]),
    "poyalgn_free": (None, [_P]),
    "poyalgn_last_error": (C.c_char_p, []),
    "poyalgn_version": (C.c_char_p, []),
    "poyalgn_cm_build": (_I, [_P, _P, _I, _I, C.POINTER(_P)]),
    "poyalgn_cm_adopt": (_I, [_P, _I, _I, _I, _I, _I, _I, _P, _P, _P, _P, _P, C.POINTER(_P)]),
    "poyalgn_cm_tables": (_I, [_P, _P, _P, _P, _P, _P, _P]),
    "poyalgn_cm_free": (None, [_P]),
    "poyalgn_simple_2": (_I, [_P, _P, _P, _I, _P, _I, _I, _P]),
    "poyalgn_backtrace_2d": (_I, [_P, _P, _P, _I, _P, _I, _P, _P, _I, _P, _I]),
    "poyalgn_align_2d": (_I, [_P, _P, _P, _I, _P, _I, _P, _P, _I, _P, _I, _I, _P]),
    "poyalgn_align_affine_3": (_I, [_P, _P, _P, _I, _P, _I, _P, _P, _P, _P, _I, _P, _I, _P]),
    "poyalgn_aligned_medians": (_I, [_P, _P, _P, _P, _I, _P, _I, _P, _P, _P]),
    "poyalgn_median_batch": (_I, [_P, _P, _I] + [_P] * 17),
    "poyalgn_verify_2": (_I, [_P, _P, _P, _P, _I, _P]),
    "poyalgn_median_2_no_gaps": (_I, [_P, _P, _P, _P, _I, _P, _I, _P]),
    "poyalgn_limit_2": (_I, [_P, _P, _P, _I, _P, _I] + [_I] * 6 + [_P]),
    "poyalgn_backtrace_2d_limit": (_I, [_P, _P, _P, _I, _P, _I, _P, _P, _I, _P] + [_I] * 5),
    "poyalgn_newkk_median_batch": (_I, [_P, _P, _I] + [_P] * 17),
    "poyalgn_newkk_median_batch_device": (_I, [_P, _P, _I] + [_P] * 6 + [_I] + [_P] * 12),
    "poyalgn_newkk_algn_affine": (_I, [_P, _P, _P, _I, _P, _I, _I, _P]),
    "poyalgn_newkk_backtrace_affine": (_I, [_P, _P, _P, _I, _P, _I, _P, _P, _I, _P, _I]),
    "poyalgn_newkk_get_k": (_I, [_P, _P]),
    "poyalgn_powell_3d": (_I, [_P, _P, _I, _P, _I, _P, _I, _I, _I, _I, _P, _P, _P, _I, _P, _P]),
    "poyalgn_powell_3d_batch": (_I, [_P, _I, _P, _P, _P, _I, _I, _I] + [_P] * 7),
    "poyalgn_powell_3d_stats": (_I, [_P, _P, _P]),
    "poyalgn_powell_3d_set_budget": (_I, [_P, _I64]),
    "poyalgn_newkk_set_arena_words": (_I, [_P, _I64]),
    "poyalgn_median_batch_device": (_I, [_P, _P, _I, _I, _I64] + [_P] * 18),
    "poyalgn_median_batch_device_noalloc": (_I, [_P, _I, _I, _I64] + [_P] * 18),
    "poyalgn_store_create": (_I, [_P, _I64, C.POINTER(_P)]),
    "poyalgn_store_free": (None, [_P]),
    "poyalgn_store_add": (_I, [_P, _P, _I, _P]),
    "poyalgn_store_count": (_I, [_P]),
    "poyalgn_store_length": (_I, [_P, _I]),
    "poyalgn_store_read": (_I, [_P, _I, _P, _I]),
    "poyalgn_store_truncate": (_I, [_P, _I]),
    "poyalgn_store_median_batch": (_I, [_P, _P, _I, _P, _P, _I, _P, _P, _P, _P]),
    "poyalgn_downpass": (_I, [_P, _P, _I, _P, _I, _P, _P, _P, _P, _P, _P]),
    "poyalgn_store_median3_batch": (_I, [_P, _P, _I, _P, _P, _P, _P, _P, _P, _P]),
    "poyalgn_uppass": (_I, [_P, _P, _I, _P, _I, _P, _P, _P, _P, _P, _P]),
    "poyalgn_store_closest_batch": (_I, [_P, _P, _I, _P, _P, _P, _P, _P]),
    "poyalgn_store_readjust_batch": (_I, [_P, _P, _I, _P, _P, _P, _P, _P, _P, _P]),
    "poyalgn_server_create": (_I, [_P, _P, _I, _I, _I, _I, _I, _I64, C.POINTER(_P)]),
    "poyalgn_server_free": (None, [_P]),
    "poyalgn_server_submit": (_I, [_P, _I, _P, _P, _P]),
    "poyalgn_server_wait": (_I, [_P, _I64, _I, _P, _P, _P, _P, _I64, _P]),
    "poyalgn_server_replay": (_I, [_P, _I, _P, _P, _P, _P, _P, _P, _P, _P]),
    "poyalgn_server_stats": (_I, [_P, _P, _P, _P]),
    "poyalgn_set_ladder": (_I, [_P, _I, _P, _P]),
    "poyalgn_get_ladder": (_I, [_P, _I, _P, _P]),
    "poyalgn_autotune": (_I, [_P, _P, _I, _P, _P, _P, _P, _P, _I, _P, _P, _I, _P, _P]),
    "poyalgn_cost_affine_3": (_I, [_P, _P, _P, _I, _P, _I, _P]),
    "poyalgn_distance_batch": (_I, [_P, _P, _I, _P, _P, _P, _P, _P, _I, _P, _P]),
    "poyalgn_distance_batch_device": (_I, [_P, _P, _I, _I, _P, _P, _P, _P, _P, _I, _P, _P, _P]),
    "poyalgn_set_row_tile": (_I, [_P, _I]),
    "poyalgn_set_speculation": (_I, [_P, _I, _I]),
    "poyalgn_set_memory_budget": (_I, [_P, _I64, _I64]),
    "poyalgn_batch_graph_create": (_I, [_P, _P, _I, _I, _I64] + [_P] * 17 + [C.POINTER(_P)]),
    "poyalgn_batch_graph_launch": (_I, [_P, _P]),
    "poyalgn_batch_graph_free": (None, [_P]),
    "poyalgn_last_launches": (_I, [_P]),
    "poyalgn_profile_begin": (_I, [_P, _I]),
    "poyalgn_profile_end": (_I, [_P, _P, _P]),
    "poyalgn_num_classes": (_I, []),
    "poyalgn_int32_peak": (_I, [_I, _I, _I, _P, _P, _P]),
}

_lib = None


def header_symbols() -> list[str]:
    """Function names declared in include/poyalgn.h."""
    text = open(HEADER).read()
    return sorted(set(re.findall(r"\b(poyalgn_[a-z0-9_]+)\s*\(", text)))


def load() -> C.CDLL:
    """Load the library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise FileNotFoundError(
            f"{LIB_PATH} is missing: build it with `python -m poy5_gb300.build` "
            "(the CUDA library is the only compute path)")
    lib = C.CDLL(LIB_PATH)
    for name, (res, args) in _SIGS.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def check(rc: int):
    if rc != 0:
        msg = load().poyalgn_last_error().decode(errors="replace")
        raise PoyAlgnError(rc, msg)
