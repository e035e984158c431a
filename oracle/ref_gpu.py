"""The reference's own generated GPU kernel, as a timed comparison point (test infrastructure:
never part of the engine, never the thing measured as this project's result).

``generate(name)`` runs where the reference tree is (path in BITGEN_REF, default the usual
checkout): it imports BitGen read-only with the stub modules of ``tests/golden/make_golden.py``,
parses each group's Pablo (this project's emitter, while-loop form, standing in for icgrep)
with the reference's ``BitstreamParser``, applies its ``run_passes``
(``bitgen/from_icgrep.py:124-166``) with ``--pass-cc-advanced=0`` (outputs at their own
positions, comparable bit for bit), ``--pass-short-circuit=0`` and ``--pass-graph-break=-1``
(one fused kernel), and lowers the groups with its ``CudaGenerator``
(``bitgen/codegen/gen_cuda.py:395-497``).  The generated ``kernel_0.cu`` (the reference's
template plus ``KernelGenerated``) is written to ``oracle/_ref/<name>.cu`` with
``<name>.json`` (block size, groups, a fingerprint of the regex groups).  Nothing generated is
committed; the files travel with the checkout.

``build(name)`` compiles that file for sm_103a with a small launcher written here (the
``cuLaunchKernel`` of ``bitgen/backend/cuda/cuda_kernel.py:411-427``: grid = (groups,
inputs), block = the configured block size) into ``oracle/_ref/lib<name>.so``.

``RefKernel(name, groups)`` binds it.  Before any launch it checks, from the generated source,
that every regex function's loop advances (its step ``blockDim.x - (offset + 32) / 32`` is at
least one word), so the kernel ends.  The generated loop loads basis words up to one block past
the end of each plane (``regex_<g>``'s ``basic_stream[idx + k * n_unit_basic]`` for ``idx <
n_unit_basic + threadIdx.x``); ``basis_buffer`` therefore allocates the planes with a zeroed
tail of one block.
"""

from __future__ import annotations

import ctypes as C
import hashlib
import json
import os
import re
import shutil
import subprocess
import sys
import tempfile
from typing import List, Sequence

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
REPO = os.path.dirname(HERE)
REF = os.environ.get("BITGEN_REF", "/root/reference")

# the DNA motif workload: 64 IUPAC motifs (seed 5) in 4 groups
DNA = "dna_64motifs_4groups"


def workload_groups(name: str) -> List[List[str]]:
    if REPO not in sys.path:
        sys.path.insert(0, REPO)
    from bitgen_gb300 import workloads
    if name == DNA:
        return [list(g) for g in workloads.dna_motifs(64, seed=5).groups(4)]
    raise KeyError(name)


def fingerprint(groups: Sequence[Sequence[str]]) -> str:
    return hashlib.sha256(json.dumps([list(g) for g in groups]).encode()).hexdigest()[:16]


LAUNCHER = r'''
extern "C" int ref_launch(const void *basis, unsigned int n_unit, unsigned int n_char,
                          void *result, void *tmp, int groups, int inputs, int block,
                          void *stream) {
  KernelGenerated<<<dim3(groups, inputs, 1), dim3(block, 1, 1), 0, (cudaStream_t)stream>>>(
      (uint32_t *)basis, n_unit, n_char, (uint32_t *)result, (uint32_t *)tmp);
  return (int)cudaGetLastError();
}
'''


def generate(name: str, block: int = 256) -> str:
    """Write oracle/_ref/<name>.cu and <name>.json from the reference's code generator."""
    groups = workload_groups(name)
    sys.path.insert(0, os.path.join(REPO, "tests", "golden"))
    import make_golden
    cfg = make_golden.import_reference()
    from bitgen import from_icgrep
    from bitgen.bitparser.bitstream_parser import BitstreamParser
    from bitgen.codegen.gen_cuda import CudaGenerator
    from bitgen_gb300.regex import compile_group

    flags = {"pass_cc_advanced": 0, "pass_cc_advanced_max": 1, "pass_cc_advanced_merge_cc": 1,
             "pass_short_circuit": 0, "pass_short_circuit_start": 2,
             "pass_short_circuit_interval": 2, "pass_short_circuit_interval_disable": 0,
             "pass_short_circuit_syncpoint": 1, "pass_graph_break": -1, "pass_print_graph": 0,
             "pass_inst_stats": 0, "pass_inst_stats_dyn": 0, "parallel_compile_cuda": False,
             "use_cached_code": False, "multi_input": 1, "block_size": (block, 1, 1),
             "backend": "cuda"}
    for k, v in flags.items():
        cfg.set_config(k, v)
    tmp = tempfile.mkdtemp(prefix="bg_refgen_")
    try:
        insts_list, maps = [], []
        for gi, g in enumerate(groups):
            path = os.path.join(tmp, f"group_{gi}.pablo")
            with open(path, "w") as f:
                f.write(compile_group(list(g), matchstar=False).to_pablo())
            p = BitstreamParser()
            insts_list.append(from_icgrep.run_passes(p.parse_file(path), p.var_name_map))
            maps.append(p.var_name_map)
        cfg.set_config("__cached_module_path", os.path.join(tmp, "module"))
        gen = CudaGenerator(insts_list, maps, [list(g) for g in groups])
        gen.lower()
        # lower() leaves both files open (gen_cuda.py:475-497): flush them before the copy
        gen.kernel_file_handler.close()
        gen.kernel_wrapper_file_handler.close()
        os.makedirs(OUT, exist_ok=True)
        dst = os.path.join(OUT, f"{name}.cu")
        shutil.copy(os.path.join(tmp, "module", "kernels", "kernel_0.cu"), dst)
        with open(os.path.join(OUT, f"{name}.json"), "w") as f:
            json.dump({"groups": len(groups), "block": block, "fingerprint": fingerprint(groups),
                       "tmp_streams": int(getattr(gen, "tmp_streams_num", 0) or 0)}, f)
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    return dst


def ensure_generated(name: str) -> bool:
    """Generate <name> where the reference tree is and the generated file is missing or was made
    for other groups; True when the generated kernel is there afterwards."""
    meta = os.path.join(OUT, f"{name}.json")
    fresh = os.path.exists(meta) and \
        json.load(open(meta)).get("fingerprint") == fingerprint(workload_groups(name))
    if not fresh and os.path.isdir(os.path.join(REF, "bitgen")):
        generate(name)
        fresh = True
    return fresh and available(name)


def available(name: str) -> bool:
    return os.path.exists(os.path.join(OUT, f"{name}.cu")) and \
        os.path.exists(os.path.join(OUT, f"{name}.json"))


def build(name: str) -> str:
    """Compile oracle/_ref/<name>.cu with the launcher into oracle/_ref/lib<name>.so."""
    src = os.path.join(OUT, f"{name}.cu")
    lib = os.path.join(OUT, f"lib{name}.so")
    if os.path.exists(lib) and os.path.getmtime(lib) >= os.path.getmtime(src):
        return lib
    unit = os.path.join(OUT, f"{name}_launch.cu")
    with open(unit, "w") as f:
        f.write(f'#include <stdint.h>\n#include <cuda_runtime.h>\n#include "{name}.cu"\n{LAUNCHER}')
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    tmp = lib + f".{os.getpid()}.tmp"
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-shared",
                    "-Xcompiler", "-fPIC", "-o", tmp, unit], check=True, capture_output=True)
    os.replace(tmp, lib)
    return lib


def loop_steps(src: str, block: int) -> List[int]:
    """Each regex function's loop step in words (generated by gen_cuda.py's lower_graph)."""
    steps = []
    for m in re.finditer(r"idx = idx \+ blockDim\.x - \(dynamic_adv_offset \+ (\d+) \+ 32\) / 32",
                         src):
        steps.append(block - (int(m.group(1)) + 32) // 32)
    return steps


class RefKernel:
    """The generated KernelGenerated of oracle/_ref/lib<name>.so, for regex groups `groups`."""

    def __init__(self, name: str, groups: Sequence[Sequence[str]]):
        self.meta = json.load(open(os.path.join(OUT, f"{name}.json")))
        if self.meta.get("fingerprint") != fingerprint(groups):
            raise ValueError(f"oracle/_ref/{name}.cu was generated for other regex groups")
        src = open(os.path.join(OUT, f"{name}.cu")).read()
        steps = loop_steps(src, self.meta["block"])
        # the advance offsets stay fixed (cc_advanced 0): dynamic_adv_offset is only reset
        writes = re.findall(r"dynamic_adv_offset\s*([-+*|]?=)(?!=)\s*([^;]*);", src)
        if len(steps) != self.meta["groups"] or min(steps) < 1 or \
                any(w != ("=", "0") for w in writes):
            raise ValueError(f"oracle/_ref/{name}.cu: a regex loop would not advance ({steps})")
        self.block = self.meta["block"]
        self.groups = self.meta["groups"]
        self.lib = C.CDLL(build(name))
        self.lib.ref_launch.restype = C.c_int
        self.lib.ref_launch.argtypes = [C.c_void_p, C.c_uint, C.c_uint, C.c_void_p, C.c_void_p,
                                        C.c_int, C.c_int, C.c_int, C.c_void_p]
        self._tmp = None

    def basis_buffer(self, inputs: int, words: int, device):
        """uint32 planes [inputs, 8, words] with a zeroed tail of one block; returns (flat
        buffer, the [1, inputs, 8, words] view of its head)."""
        import torch
        flat = torch.zeros(inputs * 8 * words + self.block, dtype=torch.uint32, device=device)
        return flat, flat[: inputs * 8 * words].view(1, inputs, 8, words)

    def launch(self, flat, inputs: int, words: int, result, stream) -> None:
        """One launch over `inputs` inputs of `words` words: result uint32 [inputs, G, words]
        (ORed into: zero it first for a fresh result)."""
        import torch
        assert flat.numel() >= inputs * 8 * words + self.block
        assert result.numel() >= inputs * self.groups * words
        if self._tmp is None:
            self._tmp = torch.zeros(self.block, dtype=torch.uint32, device=flat.device)
        rc = self.lib.ref_launch(flat.data_ptr(), words, 32 * words, result.data_ptr(),
                                 self._tmp.data_ptr(), self.groups, inputs, self.block,
                                 C.c_void_p(int(stream.cuda_stream)))
        if rc:
            raise RuntimeError(f"reference kernel launch failed with CUDA error {rc}")
