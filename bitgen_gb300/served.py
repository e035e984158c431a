"""Served scans: a continuous-batching request loop over resident pattern sets.

Compiled programs and their launch plans stay resident on the device.  Requests (an input and
the name of a pattern set) arrive over time.  Whenever a slot is free, the loop forms a batch:
requests for one pattern set, oldest first, up to a batch size and within the HBM budget.  It
copies the batch to the device on the slot's own stream, sets the plan layout asynchronously and
launches one fused scan.  Batches on different slots overlap on the GPU, and requests that
arrive while others run are admitted as soon as a slot and the budget allow.  Each request's
latency runs from its arrival to the moment its counts are back on the host.

Request payloads may live in pinned host arenas (``RequestArena``): each pattern set's requests
laid out in arrival order, 32-byte aligned, so that the oldest requests of one set, which form
a batch, are one contiguous run of the arena (two where it wraps) and reach the device with one
copy each.  Payloads elsewhere are gathered into the slot's pinned staging buffer first.

``serve_plain`` is the comparison form: one launch per request, one at a time, in arrival order.
"""

from __future__ import annotations

import os
import time
from collections import deque
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence

import numpy as np
import torch

from . import _native as N
from .engine import Inputs, Plan, Program, out_layout

ALIGN = 32


@dataclass
class Request:
    rid: int
    arrival: float          # seconds from the start of the run
    pset: str
    data: np.ndarray        # uint8


class RequestArena:
    """Pinned host memory holding request payloads back to back (32-byte aligned).  ``take(n)``
    returns the next n bytes as a numpy view, wrapping to the start when the arena is full, so
    consecutive takes are contiguous except at a wrap."""

    def __init__(self, nbytes: int, fill: Optional[np.ndarray] = None):
        self.tensor = torch.empty(nbytes, dtype=torch.uint8).pin_memory()
        self.view = self.tensor.numpy()
        if fill is not None:
            reps = -(-nbytes // fill.size)
            for i in range(reps):
                a = i * fill.size
                self.view[a:a + fill.size] = fill[:max(0, min(fill.size, nbytes - a))]
        self.at = 0
        self.base = self.view.ctypes.data

    def take(self, n: int) -> np.ndarray:
        span = -(-n // ALIGN) * ALIGN
        if span > self.view.size:
            raise ValueError("request larger than its arena")
        if self.at + span > self.view.size:
            self.at = 0
        v = self.view[self.at:self.at + n]
        self.at += span
        return v

    def offset(self, a: np.ndarray) -> int:
        """Byte offset of view `a` in the arena, or -1 when it lies elsewhere."""
        off = a.ctypes.data - self.base if a.size else -1
        return off if 0 <= off and off + a.size <= self.view.size else -1


@dataclass
class Result:
    rid: int
    latency_ms: float
    counts: np.ndarray      # int64 [n_outputs]
    streams: Optional[np.ndarray] = None


@dataclass
class _Slot:
    stream: torch.cuda.Stream
    dev_in: torch.Tensor
    host_in: torch.Tensor
    dev_counts: torch.Tensor
    host_counts: torch.Tensor
    dev_out: Optional[torch.Tensor]
    host_out: Optional[torch.Tensor]
    plans: Dict[str, Plan]
    event: torch.cuda.Event = None
    batch: List[Request] = field(default_factory=list)
    pset: str = ""
    words: List[int] = field(default_factory=list)
    offs: List[int] = field(default_factory=list)
    total: int = 0
    bytes_in_flight: int = 0


class Server:
    def __init__(self, programs: Dict[str, Program], hbm_budget: int = 120 << 30, slots: int = 4,
                 max_batch_bytes: int = 64 << 20, max_batch_inputs: int = 1024, device="cuda",
                 return_streams: bool = False, arenas: Sequence[RequestArena] = ()):
        self.programs = programs
        self.arenas = list(arenas)
        self.budget = hbm_budget
        self.max_bytes = max_batch_bytes
        self.max_inputs = max_batch_inputs
        self.return_streams = return_streams
        self.max_out = max(p.n_outputs for p in programs.values())
        words = max_batch_bytes // 32 + max_batch_inputs * 4
        # programs that merge outputs across parts need output streams even for counts
        dev_streams = return_streams or any(p.merges for p in programs.values())
        self.slots: List[_Slot] = []
        for _ in range(slots):
            plans = {}
            for name, prog in programs.items():
                if not prog.fused:
                    raise ValueError(f"pattern set {name} is not fusable")
                max_tiles = max_batch_bytes // (32 * prog.spec.tile_words) + 2 * max_batch_inputs
                plans[name] = Plan.reserve(prog, N.BG_INPUT_BYTES, max_batch_inputs, max_tiles)
            self.slots.append(_Slot(
                stream=torch.cuda.Stream(device=device),
                dev_in=torch.empty(max_batch_bytes + max_batch_inputs * ALIGN, dtype=torch.uint8, device=device),
                host_in=torch.empty(max_batch_bytes + max_batch_inputs * ALIGN, dtype=torch.uint8).pin_memory(),
                dev_counts=torch.empty((self.max_out, max_batch_inputs), dtype=torch.int64, device=device),
                host_counts=torch.empty((self.max_out, max_batch_inputs), dtype=torch.int64).pin_memory(),
                dev_out=torch.empty((self.max_out, words), dtype=torch.uint32, device=device) if dev_streams else None,
                host_out=torch.empty((self.max_out, words), dtype=torch.uint32).pin_memory() if return_streams else None,
                plans=plans))
        self.in_flight_bytes = 0
        self.copy_threads = max(1, min(8, os.cpu_count() or 1))
        self.pool = ThreadPoolExecutor(max_workers=self.copy_threads)

    # --------------------------------------------------------------------------------------
    def _runs(self, batch: List[Request]):
        """The batch as contiguous runs of one arena: [(arena, first byte, bytes, first request,
        requests)], or None when a payload lies outside every arena."""
        runs = []
        for i, r in enumerate(batch):
            where = None
            for a in self.arenas:
                off = a.offset(r.data)
                if off >= 0:
                    where = (a, off)
                    break
            if where is None:
                return None
            a, off = where
            if runs and runs[-1][0] is a and runs[-1][1] + runs[-1][2] == off:
                run = runs[-1]
                runs[-1] = (a, run[1], run[2] + -(-r.data.size // ALIGN) * ALIGN, run[3], run[4] + 1)
            else:
                runs.append((a, off, -(-r.data.size // ALIGN) * ALIGN, i, 1))
        return runs

    def _launch(self, slot: _Slot, pset: str, batch: List[Request], footprint: int):
        prog = self.programs[pset]
        offs, pos = [], 0
        for r in batch:
            offs.append(pos)
            pos += -(-r.data.size // ALIGN) * ALIGN
        lens = [int(r.data.size) for r in batch]
        out_offs, words, total = out_layout(lens)
        s = slot.stream
        sp = int(s.cuda_stream)
        runs = self._runs(batch)
        if runs is not None:
            # payloads in arenas: one host-to-device copy per contiguous run
            with torch.cuda.stream(s):
                for a, off, span, first, _ in runs:
                    at = offs[first]
                    slot.dev_in[at:at + span].copy_(a.tensor[off:off + span], non_blocking=True)
        else:
            # gather the requests into the pinned staging buffer, on several host threads for
            # large batches (numpy copies release the GIL), then one copy
            host = slot.host_in.numpy()

            def gather(lo: int, hi: int):
                for i in range(lo, hi):
                    d = batch[i].data
                    host[offs[i]:offs[i] + d.size] = d
            if pos >= (8 << 20) and len(batch) > 1:
                k = min(self.copy_threads, len(batch))
                step = -(-len(batch) // k)
                list(self.pool.map(lambda a: gather(a, min(len(batch), a + step)), range(0, len(batch), step)))
            else:
                gather(0, len(batch))
            with torch.cuda.stream(s):
                slot.dev_in[:pos].copy_(slot.host_in[:pos], non_blocking=True)
        plan = slot.plans[pset]
        plan.set_layout(Inputs(slot.dev_in, N.BG_INPUT_BYTES, offs, lens), out_offs, total, sp)
        out_ptr = slot.dev_out.data_ptr() if slot.dev_out is not None else 0
        plan.launch(slot.dev_in.data_ptr(), out_ptr, slot.dev_counts.data_ptr(), sp)
        with torch.cuda.stream(s):
            n = len(batch)
            # counts are [n_outputs][n_inputs] with row stride n for this launch
            flat = slot.dev_counts.view(-1)[:prog.n_outputs * n]
            slot.host_counts.view(-1)[:prog.n_outputs * n].copy_(flat, non_blocking=True)
            if slot.host_out is not None:
                # streams are written with row stride `total` (this batch's words)
                m = prog.n_outputs * total
                slot.host_out.view(-1)[:m].copy_(slot.dev_out.view(-1)[:m], non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(s)
        slot.event = ev
        slot.batch = batch
        slot.pset = pset
        slot.offs, slot.words, slot.total = out_offs, words, total
        slot.bytes_in_flight = footprint
        self.in_flight_bytes += footprint

    def _finish(self, slot: _Slot, now: float, results: Dict[int, Result]):
        plan = slot.plans[slot.pset]
        plan.sync(int(slot.stream.cuda_stream))  # event already complete: reports device errors
        prog = self.programs[slot.pset]
        n = len(slot.batch)
        cnt = slot.host_counts.view(-1)[:prog.n_outputs * n].numpy().reshape(prog.n_outputs, n)
        rows = None
        if slot.host_out is not None:
            rows = slot.host_out.view(-1)[:prog.n_outputs * slot.total].view(prog.n_outputs, slot.total)
        for i, r in enumerate(slot.batch):
            st = None
            if rows is not None:
                st = rows[:, slot.offs[i]:slot.offs[i] + slot.words[i]].numpy().copy()
            results[r.rid] = Result(r.rid, (now - r.arrival) * 1e3, cnt[:, i].copy(), st)
        self.in_flight_bytes -= slot.bytes_in_flight
        slot.batch = []
        slot.event = None

    def _footprint(self, pset: str, size: int) -> int:
        return size + self.programs[pset].n_outputs * (size // 8 + 16)

    def serve(self, requests: Sequence[Request], realtime: bool = True) -> Dict[int, Result]:
        """Run the request loop until every request is answered; returns results by id."""
        reqs = sorted(requests, key=lambda r: r.arrival)
        pending: Dict[str, deque] = {name: deque() for name in self.programs}
        results: Dict[int, Result] = {}
        nxt = 0
        t0 = time.perf_counter()
        while len(results) < len(reqs):
            now = time.perf_counter() - t0 if realtime else float("inf")
            while nxt < len(reqs) and reqs[nxt].arrival <= now:
                pending[reqs[nxt].pset].append(reqs[nxt])
                nxt += 1
            # completions
            for slot in self.slots:
                if slot.event is not None and slot.event.query():
                    self._finish(slot, time.perf_counter() - t0 if realtime else 0.0, results)
            # admissions: oldest waiting request first
            for slot in self.slots:
                if slot.event is not None:
                    continue
                heads = [(q[0].arrival, name) for name, q in pending.items() if q]
                if not heads:
                    break
                _, pset = min(heads)
                q = pending[pset]
                batch, size, foot = [], 0, 0
                while q and len(batch) < self.max_inputs:
                    r = q[0]
                    sz = -(-r.data.size // ALIGN) * ALIGN
                    f = self._footprint(pset, sz)
                    if batch and (size + sz > self.max_bytes or self.in_flight_bytes + foot + f > self.budget):
                        break
                    if not batch and self.in_flight_bytes + f > self.budget and self.in_flight_bytes > 0:
                        break
                    batch.append(q.popleft())
                    size += sz
                    foot += f
                if batch:
                    self._launch(slot, pset, batch, foot)
            if all(s.event is None for s in self.slots) and nxt < len(reqs) and not any(pending.values()):
                if realtime:
                    wait = reqs[nxt].arrival - (time.perf_counter() - t0)
                    if wait > 0:
                        time.sleep(min(wait, 0.002))
            elif realtime:
                time.sleep(0)
        return results


def serve_plain(programs: Dict[str, Program], requests: Sequence[Request], device="cuda",
                realtime: bool = True, arenas: Sequence[RequestArena] = ()) -> Dict[int, Result]:
    """One launch per request, one request at a time, in arrival order (payloads in `arenas`
    are copied from there, others through a pinned staging buffer)."""
    reqs = sorted(requests, key=lambda r: r.arrival)
    results: Dict[int, Result] = {}
    stream = torch.cuda.Stream(device=device)
    sp = int(stream.cuda_stream)
    biggest = max(r.data.size for r in reqs)
    dev_in = torch.empty(biggest + ALIGN, dtype=torch.uint8, device=device)
    host_in = torch.empty(biggest + ALIGN, dtype=torch.uint8).pin_memory()
    max_out = max(p.n_outputs for p in programs.values())
    dev_counts = torch.empty(max_out, dtype=torch.int64, device=device)
    host_counts = torch.empty(max_out, dtype=torch.int64).pin_memory()
    plans = {name: Plan.reserve(p, N.BG_INPUT_BYTES, 1, biggest // (32 * p.spec.tile_words) + 2)
             for name, p in programs.items()}
    t0 = time.perf_counter()
    for r in reqs:
        if realtime:
            wait = r.arrival - (time.perf_counter() - t0)
            if wait > 0:
                time.sleep(wait)
        prog = programs[r.pset]
        src = None
        for a in arenas:
            off = a.offset(r.data)
            if off >= 0:
                src = a.tensor[off:off + r.data.size]
                break
        if src is None:
            host_in.numpy()[:r.data.size] = r.data
            src = host_in[:r.data.size]
        with torch.cuda.stream(stream):
            dev_in[:r.data.size].copy_(src, non_blocking=True)
        offs, words, total = out_layout([r.data.size])
        plans[r.pset].set_layout(Inputs(dev_in, N.BG_INPUT_BYTES, [0], [int(r.data.size)]), offs, total, sp)
        plans[r.pset].launch(dev_in.data_ptr(), 0, dev_counts.data_ptr(), sp)
        with torch.cuda.stream(stream):
            host_counts[:prog.n_outputs].copy_(dev_counts[:prog.n_outputs], non_blocking=True)
        plans[r.pset].sync(sp)
        now = time.perf_counter() - t0
        results[r.rid] = Result(r.rid, (now - r.arrival) * 1e3, host_counts[:prog.n_outputs].numpy().copy())
    return results


def latency_stats(results: Dict[int, Result]) -> dict:
    lat = np.array([r.latency_ms for r in results.values()])
    return {"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "mean_ms": float(lat.mean()), "n": int(lat.size)}
