"""ctypes binding of ``libbitgen_gb300.so`` (the C ABI in ``include/bitgen_gb300.h``).

The library is built in-tree by :func:`bitgen_gb300.build.build`.  There is no fallback: if the
library is missing or cannot be loaded, :func:`lib` raises, so no scan ever runs on anything but
the native GPU path.
"""

from __future__ import annotations

import ctypes as C
import os
import threading

from .build import LIB

BG_OK, BG_ERR_INVALID, BG_ERR_CUDA, BG_ERR_COMPILE, BG_ERR_TIMEOUT, BG_ERR_ALIGN, BG_ERR_NOMEM, BG_ERR_DEVICE, BG_ERR_CAPACITY = range(9)
BG_INPUT_BYTES, BG_INPUT_BASIS = 0, 1
BG_PROGRAM_MERGES = 1

_lock = threading.Lock()
_lib = None


class BitgenError(RuntimeError):
    def __init__(self, status: int, what: str, detail: str = ""):
        self.status = status
        msg = f"{what}: {status_string(status)}"
        if detail:
            msg += f" ({detail})"
        super().__init__(msg)


class KernelDesc(C.Structure):
    _fields_ = [("source", C.c_char_p), ("source_len", C.c_size_t), ("name", C.c_char_p),
                ("n_outputs", C.c_int32), ("n_adds", C.c_int32), ("halo_lanes", C.c_int32),
                ("wpt", C.c_int32), ("block", C.c_int32), ("tail_lanes", C.c_int32),
                ("n_pre", C.c_int32), ("n_run", C.c_int32), ("flags", C.c_int32),
                ("n_parts", C.c_int32)]


class Layout(C.Structure):
    _fields_ = [("input_kind", C.c_int32), ("n_inputs", C.c_int32),
                ("in_off", C.POINTER(C.c_int64)), ("in_len", C.POINTER(C.c_int64)),
                ("basis_stride", C.c_int64), ("out_off", C.POINTER(C.c_int64)),
                ("out_stride", C.c_int64)]


class Instr(C.Structure):
    _fields_ = [("op", C.c_int32), ("dst", C.c_int32), ("a", C.c_int32), ("b", C.c_int32),
                ("c", C.c_int32), ("shift", C.c_int32)]


# name -> (restype, argtypes); mirrors include/bitgen_gb300.h
SIGNATURES = {
    "bg_status_string": (C.c_char_p, [C.c_int]),
    "bg_last_error": (C.c_char_p, []),
    "bg_device_available": (C.c_int, []),
    "bg_transpose": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_int64, C.c_void_p]),
    "bg_program_create": (C.c_int, [C.POINTER(KernelDesc), C.POINTER(C.c_void_p)]),
    "bg_nvrtc_check": (C.c_int, [C.c_char_p, C.c_size_t, C.c_char_p, C.c_char_p, C.c_size_t]),
    "bg_program_log": (C.c_int, [C.c_void_p, C.c_char_p, C.c_size_t]),
    "bg_program_info": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                  C.POINTER(C.c_int32)]),
    "bg_program_destroy": (C.c_int, [C.c_void_p]),
    "bg_plan_create": (C.c_int, [C.c_void_p, C.POINTER(Layout), C.POINTER(C.c_void_p)]),
    "bg_plan_reserve": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int64, C.POINTER(C.c_void_p)]),
    "bg_plan_set_layout": (C.c_int, [C.c_void_p, C.POINTER(Layout), C.c_void_p]),
    "bg_plan_tiles": (C.c_int64, [C.c_void_p]),
    "bg_plan_set_wait_limit": (C.c_int, [C.c_void_p, C.c_int64, C.c_int64]),
    "bg_plan_set_positions": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64]),
    "bg_plan_positions_written": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(C.c_int64)]),
    "bg_plan_stats": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.POINTER(C.c_int64),
                              C.POINTER(C.c_int64)]),
    "bg_plan_launch": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "bg_plan_sync": (C.c_int, [C.c_void_p, C.c_void_p]),
    "bg_plan_destroy": (C.c_int, [C.c_void_p]),
    "bg_scan_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_int64,
                                  C.c_void_p, C.c_void_p, C.c_void_p]),
    "bg_interp_create": (C.c_int, [C.POINTER(Instr), C.c_int32, C.c_int32, C.POINTER(C.c_int32),
                                   C.c_int32, C.POINTER(C.c_void_p)]),
    "bg_interp_run": (C.c_int, [C.c_void_p, C.POINTER(Layout), C.c_void_p, C.c_void_p, C.c_void_p,
                                C.c_int64, C.c_void_p]),
    "bg_interp_destroy": (C.c_int, [C.c_void_p]),
}


def lib():
    """Load (once) and return the native library; raises if it is not built."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB):
                raise RuntimeError(
                    f"native library {LIB} is missing: build it with "
                    "`python -c 'import __graft_entry__ as g; g.build()'` or "
                    "`python -m bitgen_gb300.build`")
            L = C.CDLL(LIB)
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


def status_string(status: int) -> str:
    try:
        return lib().bg_status_string(status).decode()
    except Exception:  # pragma: no cover - only when the library itself is absent
        return str(status)


def check(status: int, what: str):
    if status != BG_OK:
        detail = lib().bg_last_error().decode(errors="replace")
        raise BitgenError(status, what, detail)
