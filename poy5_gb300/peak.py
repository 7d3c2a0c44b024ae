"""Measured integer issue rates of this GPU (poyalgn_int32_peak).

The fill kernels are bound by integer instruction issue, so their roofline
is reported against these measured rates, not a nominal lane count.
"""
from __future__ import annotations

import ctypes as C

from . import _lib

KINDS = {"add": 0, "min": 1, "logic": 2, "min3_dpx": 3, "max3_u16x2_dpx": 4}
# single-operation instruction kinds: the roofline peak is the fastest
SINGLE_OP = ("add", "min", "logic")


def int32_rates(device: int = 0, iters: int = 20000) -> dict:
    """Thread-instructions per second of each kind, and the roofline peak
    (the fastest single-operation kind) in Tops."""
    lib = _lib.load()
    out = {}
    for name, kind in KINDS.items():
        rate, ms, n = C.c_double(), C.c_float(), C.c_int64()
        _lib.check(lib.poyalgn_int32_peak(device, kind, iters, C.byref(rate), C.byref(ms),
                                          C.byref(n)))
        out[name] = {"tinst_per_s": rate.value / 1e12, "ms": ms.value, "thread_inst": n.value}
    best = max(SINGLE_OP, key=lambda k: out[k]["tinst_per_s"])
    return {"kinds": out, "peak_tops": out[best]["tinst_per_s"], "peak_kind": best}
