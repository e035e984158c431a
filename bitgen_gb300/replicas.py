"""Multi-GPU form of the scan: independent replicas, no collective on the data path.

The reference has no multi-GPU code (its parallelism is regex groups x replicated inputs inside
one kernel, ``bitgen/codegen/gen_cuda.py:411-413``).  Scans shard by input: every rank scans its
own inputs (or its own replica of the benchmark input), and the only cross-rank traffic is the
timing reduction around the measured region (a barrier and a max over ranks).
"""

from __future__ import annotations

import os
from typing import List, Sequence

import torch
import torch.distributed as dist


def world() -> tuple:
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), \
        int(os.environ.get("LOCAL_RANK", "0"))


def init(backend: str, device=None):
    rank, size, _ = world()
    if size > 1 and not dist.is_initialized():
        if device is not None and backend == "nccl":
            dist.init_process_group(backend, device_id=device)
        else:
            dist.init_process_group(backend)
    return rank, size


def shard(items: Sequence, rank: int, size: int) -> List:
    """Round-robin partition of independent inputs over ranks."""
    return [x for i, x in enumerate(items) if i % size == rank]


def barrier():
    if dist.is_initialized():
        dist.barrier()


def max_over_ranks(values: Sequence[float], device=None) -> List[float]:
    """Element-wise max of per-rank values (e.g. step times) across all ranks."""
    t = torch.tensor(list(values), dtype=torch.float64, device=device)
    if dist.is_initialized() and dist.get_world_size() > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t.tolist()]
