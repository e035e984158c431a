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


def reach(code) -> "tuple[int, int] | None":
    """(back, ahead): how many characters before and after a position the outputs of a flat
    program can depend on, or None when the program has additions or loops (MatchStar,
    ScanThru, while, if), whose reach is unbounded."""
    back: dict = {}
    ahead: dict = {}
    for op, dst, a, b, c, shift in code:
        if op in (6, 7, 9, 10):
            return None
        srcs = [x for x in (a, b, c) if x >= 0]
        bk = max([back.get(x, 0) for x in srcs] + [0])
        ah = max([ahead.get(x, 0) for x in srcs] + [0])
        if op == 5:
            bk += shift
        elif op == 11:
            ah += shift
        back[dst], ahead[dst] = bk, ah
    return max(list(back.values()) + [0]), max(list(ahead.values()) + [0])


def run_groups(groups, data: np.ndarray, per_regex: bool = False, threads: int = 0,
               max_iter: int = 0, split: bool = False):
    """Evaluate Pablo groups over one input on the host.  Returns (list of uint32 streams,
    counts).  By default each group runs on its own thread.  With ``split`` and programs of
    bounded reach (no additions or loops, see `reach`), the input is instead cut into one
    byte range per thread, each range evaluated with enough bytes before and after it to
    cover that reach, so that every thread works whatever the number of groups; the stitched
    streams equal the unsplit ones."""
    from bitgen_gb300.engine import lower_interp

    progs = [lower_interp([g], per_regex) for g in groups]
    threads = threads or os.cpu_count() or 1
    reaches = [reach(p[0]) for p in progs]
    n = int(data.size)
    if split and threads > 1 and all(r is not None for r in reaches) and n >= 64 * threads:
        back = max(r[0] for r in reaches)
        ahead = max(r[1] for r in reaches)
        hb = -(-back // 64) * 64           # whole 64-byte words before a range
        cuts = [min(n, (n * i // threads) // 64 * 64) for i in range(threads)] + [n]
        W = (n + 31) // 32

        def one(i):
            lo, hi = cuts[i], cuts[i + 1]
            a, b = max(0, lo - hb), min(n, hi + ahead)
            outs = [run_code(p[0], p[1], p[2], data[a:b], max_iter)[0] for p in progs]
            return lo, hi, a, outs

        with ThreadPoolExecutor(max_workers=threads) as ex:
            parts = list(ex.map(one, range(threads)))
        streams = [np.zeros(W, dtype=np.uint32) for p in progs for _ in p[2]]
        for lo, hi, a, outs in parts:
            if hi <= lo:
                continue
            w0, w1, skip = lo // 32, (hi + 31) // 32, (lo - a) // 32
            k = 0
            for o in outs:
                for row in o:
                    streams[k][w0:w1] = row[skip:skip + w1 - w0]
                    k += 1
        counts = [int(np.bitwise_count(s).sum(dtype=np.int64)) for s in streams]
        return streams, counts
    with ThreadPoolExecutor(max_workers=max(1, min(threads, len(progs)))) as ex:
        res = list(ex.map(lambda p: run_code(p[0], p[1], p[2], data, max_iter), progs))
    streams: List[np.ndarray] = []
    counts: List[int] = []
    for s, c in res:
        streams.extend(list(s))
        counts.extend(int(x) for x in c)
    return streams, counts
