"""ctypes wrapper of the C word-parallel oracle ``bg_cpu.c`` (test infrastructure only).

``build()`` compiles it with gcc into ``oracle/_build/libbg_cpu.so``.  ``run_groups`` evaluates
Pablo groups over one input on the host, one group per thread, and returns the output streams in
the reference layout plus popcounts.  It is the full-size parity checker for the GPU path and
the timed CPU baseline (standing in for icgrep, which is not available).
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading
from concurrent.futures import ThreadPoolExecutor
from typing import List, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "bg_cpu.c")
OUT = os.path.join(HERE, "_build", "libbg_cpu.so")
_lock = threading.Lock()
_lib = None


class Instr(C.Structure):
    _fields_ = [("op", C.c_int32), ("dst", C.c_int32), ("a", C.c_int32), ("b", C.c_int32),
                ("c", C.c_int32), ("shift", C.c_int32)]


def build(force: bool = False) -> str:
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    if force or not os.path.exists(OUT) or os.path.getmtime(OUT) < os.path.getmtime(SRC):
        tmp = OUT + f".{os.getpid()}.tmp"
        subprocess.run(["gcc", "-O3", "-fPIC", "-shared", "-std=c11", "-o", tmp, SRC], check=True)
        os.replace(tmp, OUT)
    return OUT


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = C.CDLL(OUT)
            L.bgc_run.restype = C.c_int
            L.bgc_run.argtypes = [C.POINTER(Instr), C.c_int, C.c_int, C.POINTER(C.c_int), C.c_int,
                                  C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_int64, C.c_int64]
            _lib = L
    return _lib


def run_code(code, n_slots: int, outs: Sequence[int], data: np.ndarray, max_iter: int = 0,
             block_words: int = 256):
    """Run one flat program; returns (uint32 [n_out, W32], uint64 [n_out])."""
    data = np.ascontiguousarray(data, dtype=np.uint8)
    n = data.size
    W32 = (n + 31) // 32
    arr = (Instr * max(1, len(code)))(*[Instr(*c) for c in code])
    o = (C.c_int * max(1, len(outs)))(*outs)
    out = np.zeros((len(outs), max(W32, 1)), dtype=np.uint32)
    cnt = np.zeros(len(outs), dtype=np.uint64)
    rc = lib().bgc_run(arr, len(code), n_slots, o, len(outs), data.ctypes.data, n,
                       out.ctypes.data, cnt.ctypes.data, max_iter, block_words)
    if rc != 0:
        raise RuntimeError(f"bgc_run failed with status {rc}")
    return out[:, :W32], cnt


def run_groups(groups, data: np.ndarray, per_regex: bool = False, threads: int = 0,
               max_iter: int = 0):
    """Evaluate each group on its own thread.  Returns (list of uint32 streams, counts)."""
    from bitgen_gb300.engine import lower_interp

    progs = [lower_interp([g], per_regex) for g in groups]
    threads = threads or os.cpu_count() or 1
    with ThreadPoolExecutor(max_workers=max(1, min(threads, len(progs)))) as ex:
        res = list(ex.map(lambda p: run_code(p[0], p[1], p[2], data, max_iter), progs))
    streams: List[np.ndarray] = []
    counts: List[int] = []
    for s, c in res:
        streams.extend(list(s))
        counts.extend(int(x) for x in c)
    return streams, counts
