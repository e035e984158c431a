"""Batched scans: thousands of inputs of uneven length in one persistent launch.

All inputs are packed into one device buffer at 32-byte aligned offsets; one launch of the
fused kernel walks every tile of every input (the tile table maps a claimed tile to its input),
and the launch is captured once into a CUDA graph and replayed.  ``scan_per_input`` is the plain
form the batched form is compared with: one launch per input, as BitGen's runner issues one
``run_fn`` per input (``bitgen/from_icgrep.py:575-582``).
"""

from __future__ import annotations

from typing import List, Optional, Sequence

import numpy as np
import torch

from . import _native as N
from .engine import Inputs, Plan, Program, bytes_input, out_layout, pack_bytes


class BatchScanner:
    """One persistent launch over a fixed batch layout, optionally replayed as a CUDA graph."""

    def __init__(self, program: Program, items: Sequence, device="cuda", graph: bool = True,
                 streams: bool = True):
        if not program.fused:
            raise ValueError("batched scans need a fused program")
        self.program = program
        self.inp = pack_bytes(items, device=device)
        self.offs, self.words, self.total = out_layout(self.inp.lengths)
        n_out = program.n_outputs
        # a program that merges outputs across parts needs output streams even for counts
        self.out = (torch.empty((n_out, self.total), dtype=torch.uint32, device=device)
                    if streams or program.merges else None)
        self.counts = torch.empty((n_out, self.inp.n), dtype=torch.int64, device=device)
        self.plan = Plan(program, self.inp, self.offs, self.total)
        self.stream = torch.cuda.Stream(device=device)
        self.graph = None
        self._launch()          # warm up (first launch loads the module on this stream)
        self.sync()
        if graph:
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g, stream=self.stream):
                self._launch()
            self.graph = g

    def _launch(self):
        s = torch.cuda.current_stream() if torch.cuda.is_current_stream_capturing() else self.stream
        self.plan.launch(self.inp.data.data_ptr(), self.out.data_ptr() if self.out is not None else 0,
                         self.counts.data_ptr(), int(s.cuda_stream))

    def run(self):
        if self.graph is not None:
            with torch.cuda.stream(self.stream):
                self.graph.replay()
        else:
            self._launch()

    def sync(self):
        self.plan.sync(int(self.stream.cuda_stream))

    def stream_of(self, output: int, i: int) -> torch.Tensor:
        return self.out[output, self.offs[i]:self.offs[i] + self.words[i]]


class PerInputScanner:
    """The plain form: one launch (and one plan) per input, on one stream."""

    def __init__(self, program: Program, items: Sequence, device="cuda", streams: bool = True):
        self.program = program
        self.inp = pack_bytes(items, device=device)
        self.offs, self.words, self.total = out_layout(self.inp.lengths)
        n_out = program.n_outputs
        # one shared output (each input's launch writes its own words), also for counts only
        self.out = (torch.empty((n_out, self.total), dtype=torch.uint32, device=device)
                    if streams or program.merges else None)
        self.counts = torch.empty((n_out, self.inp.n), dtype=torch.int64, device=device)
        self.stream = torch.cuda.Stream(device=device)
        self.plans: List[Plan] = []
        self.views = []
        for i, (o, n) in enumerate(zip(self.inp.offsets, self.inp.lengths)):
            view = Inputs(self.inp.data, N.BG_INPUT_BYTES, [o], [n])
            # each per-input launch writes its own slice of the shared output and counts
            self.plans.append(Plan(program, view, [self.offs[i]], self.total))
            self.views.append(view)
        self.tmp_counts = torch.empty((len(self.plans), n_out, 1), dtype=torch.int64, device=device)

    def run(self):
        sp = int(self.stream.cuda_stream)
        base = self.inp.data.data_ptr()
        out = self.out.data_ptr() if self.out is not None else 0
        for i, p in enumerate(self.plans):
            p.launch(base, out, self.tmp_counts[i].data_ptr(), sp)

    def sync(self):
        sp = int(self.stream.cuda_stream)
        for p in self.plans:
            p.sync(sp)
        self.counts.copy_(self.tmp_counts[:, :, 0].T)

    def stream_of(self, output: int, i: int) -> torch.Tensor:
        return self.out[output, self.offs[i]:self.offs[i] + self.words[i]]
