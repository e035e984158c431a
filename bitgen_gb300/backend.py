"""Drop-in for BitGen's CUDA backend interface.

BitGen's runner reaches the GPU through two Python-level calls, both mirrored here with the same
names, argument meaning and return shapes:

* ``byte_stream_transpose(bytestream, bitstream)`` - the torch extension op
  (``bitgen/template/cuda/pybind.cpp:9``, ``kernel.cu:102-124``), called from
  ``bitgen/bitstream.py:199,203``: ``uint8 [S, M, Npad]`` -> caller-allocated
  ``uint32 [S, M, 8, Npad/32]``, synchronous.  Errors raise instead of ``exit()``.
* ``init_kernel(regex_func_num, input_stream_tensor, basic_stream_tensor, cfg)`` - the function
  of the generated ``kernels/kernel_0.py`` (``bitgen/backend/cuda/template/template.py:124-149``)
  that ``bitgen/from_icgrep.py:169-193`` imports.  It returns
  ``(result, tmp_streams, kernel_handle, run_fn, dyn_stats)``: ``result`` is
  ``uint32 [S, M, G, W]``; ``run_fn(basis)`` scans the basis tensor and writes ``result``;
  ``kernel_handle.free()`` releases the program.  ``tmp_streams`` is ``None`` (the fused engine
  needs no global scratch streams).  ``dyn_stats`` is ``None`` unless the configuration sets
  ``pass_inst_stats_dyn`` (the reference then builds from
  ``bitgen/backend/cuda/template/template_dyn_stat.py:39-87`` and its runner sums
  ``dyn_stats[..., :1]`` and ``dyn_stats[..., 1:]``, ``from_icgrep.py:619-640``):
  here it is ``int64 [S, 1, P, 2]``, refreshed by every ``run_fn`` call, with per part of the
  program (P = 1 for a single-kernel program) ``[..., 0]`` = the tiles it ran on (the
  reference: tile-loop iterations) and ``[..., 1]`` = the 32-tile rows of its work list (the
  reference: per-iteration advance offsets).  The reference kernel ORs into ``result``
  and relies on the caller zeroing it (``from_icgrep.py:546-552``); this engine writes it with
  plain stores, so zeroing is harmless but not needed.

``write_kernel_module`` writes such a ``kernels/kernel_0.py`` for a list of groups, the file the
reference's ``CudaGenerator.lower`` produces (``bitgen/codegen/gen_cuda.py:475-497``).
"""

from __future__ import annotations

import json
import os
from typing import List, Optional, Sequence

import torch

from .compiler import Tuning
from .engine import Program, basis_input, transpose
from .pablo import Group


def byte_stream_transpose(bytestream: torch.Tensor, bitstream: torch.Tensor) -> None:
    if bytestream.dim() != 3 or bitstream.dim() != 4 or bitstream.size(2) != 8:
        raise ValueError("byte_stream_transpose expects [S, M, Npad] -> [S, M, 8, Npad/32]")
    transpose(bytestream, bitstream)
    torch.cuda.current_stream().synchronize()


class KernelHandle:
    """What ``CUDA_Kernel`` offers the runner: ``free()`` (cuda_kernel.py:400-406)."""

    def __init__(self, program: Program):
        self.program = program

    def free(self):
        if self.program is not None:
            self.program.close()
            self.program = None


def _cfg_flag(cfg, key: str) -> bool:
    """A flag of the runner's configuration: the reference's config module
    (``bitgen/config.py:19``, ``get_config(key)`` gives None for an unset key), any object with
    such a ``get_config``, or a plain dict."""
    if cfg is None:
        return False
    if hasattr(cfg, "get_config"):
        try:
            return bool(cfg.get_config(key))
        except (KeyError, AttributeError):
            return False
    return bool(cfg.get(key)) if isinstance(cfg, dict) else False


def init_kernel(regex_func_num: int, input_stream_tensor, basic_stream_tensor: torch.Tensor,
                cfg: Optional[dict] = None, groups: Optional[Sequence[Group]] = None,
                tuning: Optional[Tuning] = None):
    """Compile ``groups`` and bind them to ``basic_stream_tensor``'s shape."""
    if groups is None:
        raise ValueError("init_kernel needs the compiled groups (write_kernel_module embeds them)")
    if len(groups) != regex_func_num:
        raise ValueError(f"{regex_func_num} regex functions requested, {len(groups)} groups given")
    if basic_stream_tensor.dim() != 4 or basic_stream_tensor.size(2) != 8:
        raise ValueError("basic_stream_tensor must be uint32 [S, M, 8, W]")
    S, M, _, W = basic_stream_tensor.shape
    if S != 1:
        raise ValueError("split_input must be 1 (bitgen/backend/cuda/template/template.py:25)")
    G = len(groups)
    program = Program(list(groups), tuning=tuning)
    result = torch.zeros((S, M, G, W), dtype=torch.uint32, device=basic_stream_tensor.device)
    out_offsets = [m * G * W for m in range(M)]
    dyn_stats = None
    if _cfg_flag(cfg, "pass_inst_stats_dyn"):
        P = max(1, program.spec.n_parts) if program.fused else 1
        dyn_stats = torch.zeros((S, 1, P, 2), dtype=torch.int64, device=basic_stream_tensor.device)

    def run_fn(basis: torch.Tensor):
        inp = basis_input(basis)
        res = program.scan(inp, streams=True, counts=False, out=result, out_offsets=out_offsets,
                           out_stride=W, stats=dyn_stats is not None)
        st = res.stats
        if st is not None and st["form"] == "split":
            dyn_stats[0, 0].copy_(torch.tensor(list(zip(st["tiles_run"], st["rows"])), dtype=torch.int64))
        elif st is not None:
            dyn_stats[0, 0, 0, 0] = st["tiles"]
        return None

    return result, None, KernelHandle(program), run_fn, dyn_stats


_MODULE = '''"""Generated by bitgen_gb300.backend.write_kernel_module (drop-in kernels/kernel_0.py)."""
import json, os
from bitgen_gb300.backend import init_kernel as _init
from bitgen_gb300.pablo import parse_pablo

_HERE = os.path.dirname(os.path.abspath(__file__))
with open(os.path.join(_HERE, "groups.json")) as _f:
    _GROUPS = [parse_pablo(t) for t in json.load(_f)]


def init_kernel(regex_func_num, input_stream_tensor, basic_stream_tensor=None, cfg={}):
    return _init(regex_func_num, input_stream_tensor, basic_stream_tensor, cfg, groups=_GROUPS)
'''


def write_kernel_module(groups: Sequence[Group], cache_dir: str) -> str:
    """Write ``<cache_dir>/kernels/{__init__,kernel_0}.py`` + ``groups.json``; return the path of
    ``kernel_0.py`` (what ``compile_regex_group_list`` returns, ``from_icgrep.py:446-525``)."""
    kdir = os.path.join(cache_dir, "kernels")
    os.makedirs(kdir, exist_ok=True)
    with open(os.path.join(kdir, "__init__.py"), "w") as f:
        f.write("from . import kernel_0\n")
    with open(os.path.join(kdir, "groups.json"), "w") as f:
        json.dump([g.to_pablo() for g in groups], f)
    path = os.path.join(kdir, "kernel_0.py")
    with open(path, "w") as f:
        f.write(_MODULE)
    return path
