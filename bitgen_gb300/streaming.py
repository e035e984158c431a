"""Double-buffered scanning of host buffers: the copy of the next buffer to the device overlaps
the scan of the current one.

A scan of one input is a host-to-device copy, the scan kernels and the read-back of the match
counts.  Run one after another, the copy (about 200 GB/s from pinned host memory) and the scan
add up; `StreamScanner` keeps two device buffers and puts the copies on their own streams, so
that in a sequence of inputs each step costs the longer of the two.  Every step still copies its
own input and reads back its own counts; nothing is cached between steps.

    sc = StreamScanner(program, n_bytes, device)
    handles = [sc.submit(buf) for buf in pinned_host_buffers]
    counts = [sc.counts(h) for h in handles]       # waits for each step

This is the streaming form of `Program.scan`: the same plan, kernels and results, bit for bit.
"""

from __future__ import annotations

from typing import List, Optional

import torch

from .engine import Plan, Program, bytes_input, out_layout


class StreamScanner:
    """Scans equally sized inputs of `n_bytes` bytes given as pinned host uint8 tensors."""

    def __init__(self, program: Program, n_bytes: int, device: torch.device,
                 copy_streams: int = 2, streams_out: bool = True):
        self.prog = program
        self.n = int(n_bytes)
        self.dev = torch.device(device)
        self.bufs = [torch.empty(self.n, dtype=torch.uint8, device=self.dev) for _ in range(2)]
        offs, words, total = out_layout([self.n])
        self.out = (torch.empty((program.n_outputs, total), dtype=torch.uint32, device=self.dev)
                    if streams_out or program.merges else None)
        self.d_counts = torch.empty((program.n_outputs, 1), dtype=torch.int64, device=self.dev)
        self.h_counts = [torch.empty((program.n_outputs, 1), dtype=torch.int64).pin_memory()
                         for _ in range(2)]
        # its own plan (look-back records, run masks, work list): scans of the same layout
        # elsewhere do not share this scratch
        self.plan = Plan(program, bytes_input(self.bufs[0]), offs, total)
        self.compute = torch.cuda.Stream(device=self.dev)
        self.copies = [torch.cuda.Stream(device=self.dev) for _ in range(max(1, copy_streams))]
        self.copied = [[torch.cuda.Event() for _ in self.copies] for _ in range(2)]
        self.done: List[Optional[torch.cuda.Event]] = [None, None]
        self.step = 0

    def submit(self, host: torch.Tensor) -> int:
        """Enqueue the copy, scan and count read-back of one input; returns a handle."""
        if host.numel() != self.n or host.dtype != torch.uint8:
            raise ValueError(f"StreamScanner: expected {self.n} uint8 bytes")
        slot = self.step & 1
        dst = self.bufs[slot]
        chunk = -(-self.n // len(self.copies))
        for i, s in enumerate(self.copies):
            a, b = i * chunk, min(self.n, (i + 1) * chunk)
            if self.done[slot] is not None:
                s.wait_event(self.done[slot])   # the scan two steps back has read this buffer
            if a < b:
                with torch.cuda.stream(s):
                    dst[a:b].copy_(host[a:b], non_blocking=True)
            self.copied[slot][i].record(s)
        c = self.compute
        for ev in self.copied[slot]:
            c.wait_event(ev)
        self.plan.launch(dst.data_ptr(), self.out.data_ptr() if self.out is not None else 0,
                         self.d_counts.data_ptr(), c.cuda_stream)
        with torch.cuda.stream(c):
            self.h_counts[slot].copy_(self.d_counts, non_blocking=True)
        ev = torch.cuda.Event()
        ev.record(c)
        self.done[slot] = ev
        self.step += 1
        return self.step - 1

    def counts(self, handle: int) -> List[int]:
        """Match counts per output of step `handle` (one of the last two submitted)."""
        if handle < self.step - 2 or handle >= self.step:
            raise ValueError("StreamScanner: only the last two steps' counts are kept")
        slot = handle & 1
        self.done[slot].synchronize()
        return [int(x) for x in self.h_counts[slot][:, 0].tolist()]

    def synchronize(self):
        for ev in self.done:
            if ev is not None:
                ev.synchronize()
