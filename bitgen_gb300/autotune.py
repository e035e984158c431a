"""Autotuner for the fused scan: words per lane, CTA size, part size, register budget.

For a pattern set and a sample input it compiles each candidate tuning, times a few launches
with CUDA events, and keeps the fastest.  Outputs never depend on the tuning (the parity tests
check that), so the choice is only about speed.  Choices are cached in
``$BG_CACHE_DIR/autotune.json``, keyed by a hash of the programs and of the sample's shape.
"""

from __future__ import annotations

import hashlib
import json
import os
from dataclasses import asdict
from typing import List, Optional, Sequence, Tuple

import torch

from .compiler import Tuning
from .engine import Inputs, Program, _ensure_cache_dir, out_layout
from .pablo import Group

SPACE = [
    Tuning(),                                              # split form, merged 2-term parts
    Tuning(part_cap=1),
    Tuning(part_cap=4, exec_groups=8),
    Tuning(merge_outputs=False, part_cap=32),              # parts of whole outputs
    Tuning(single_wpt=2, single_min_blocks=1, chain_batch=8),  # unselective sets: 2 words
                                                           # per lane, 255 registers
    Tuning(wpt=1, min_blocks=4, prefilter=False),          # single-kernel form forced
]


def _key(groups: Sequence[Group], inp: Inputs, per_regex: bool) -> str:
    h = hashlib.sha256()
    for g in groups:
        h.update(g.to_pablo().encode())
    h.update(repr((inp.kind, len(inp.lengths), sum(inp.lengths) // (1 << 20), per_regex)).encode())
    return h.hexdigest()[:24]


def _cache_path() -> str:
    _ensure_cache_dir()
    return os.path.join(os.environ["BG_CACHE_DIR"], "autotune.json")


def time_program(prog: Program, inp: Inputs, reps: int = 3) -> float:
    offs, words, total = out_layout(inp.lengths)
    out = torch.empty((prog.n_outputs, total), dtype=torch.uint32, device=inp.data.device)
    cnt = torch.empty((prog.n_outputs, inp.n), dtype=torch.int64, device=inp.data.device)
    plan = prog.plan(inp, offs, total)
    s = torch.cuda.current_stream()
    sp = int(s.cuda_stream)
    plan.launch(inp.data.data_ptr(), out.data_ptr(), cnt.data_ptr(), sp)
    plan.sync(sp)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(reps):
        plan.launch(inp.data.data_ptr(), out.data_ptr(), cnt.data_ptr(), sp)
    e1.record(s)
    plan.sync(sp)
    return e0.elapsed_time(e1) / reps


def autotune(groups: Sequence[Group], sample: Inputs, space: Optional[List[Tuning]] = None,
             per_regex: bool = False, reps: int = 3, use_cache: bool = True) -> Tuple[Tuning, list]:
    """Return (best tuning, [(tuning dict, ms), ...])."""
    space = space or SPACE
    key = _key(groups, sample, per_regex)
    path = _cache_path()
    cache = {}
    if use_cache and os.path.exists(path):
        try:
            cache = json.load(open(path))
        except (OSError, ValueError):
            cache = {}
        if key in cache:
            fields = {k: tuple(v) if isinstance(v, list) else v     # JSON keeps tuples as lists
                      for k, v in cache[key]["tuning"].items()}
            return Tuning(**fields), cache[key]["report"]
    report = []
    best, best_ms = None, float("inf")
    for t in space:
        try:
            prog = Program(list(groups), per_regex=per_regex, tuning=t, executor="fused")
        except Exception as e:  # a candidate that does not fit (e.g. halo too deep) is skipped
            report.append((asdict(t), None, str(e)[:120]))
            continue
        ms = time_program(prog, sample, reps)
        prog.close()
        report.append((asdict(t), round(ms, 4), ""))
        if ms < best_ms:
            best, best_ms = t, ms
    if best is None:
        raise RuntimeError("no candidate tuning compiled")
    cache[key] = {"tuning": asdict(best), "report": report}
    tmp = path + f".{os.getpid()}.tmp"
    with open(tmp, "w") as f:
        json.dump(cache, f, indent=1)
    os.replace(tmp, path)
    return best, report
