"""CPU: the reference's generated DNA kernel (oracle/ref_gpu.py) is generated for the workload's
groups, and its loops provably end before it is ever launched."""

import json
import os

import pytest

from oracle import ref_gpu


def test_loop_steps_parse_the_generated_loop_header():
    src = ("for (uint32_t idx = threadIdx.x; idx < n_unit_basic + threadIdx.x; "
           "idx = idx + blockDim.x - (dynamic_adv_offset + 211 + 32) / 32) {")
    assert ref_gpu.loop_steps(src, 256) == [256 - 7]
    # a reach of a whole block would leave the loop standing still
    assert ref_gpu.loop_steps(src.replace("211", str(256 * 32)), 256) == [-1]


def test_fingerprint_tracks_the_groups():
    g = ref_gpu.workload_groups(ref_gpu.DNA)
    assert len(g) == 4 and sum(len(x) for x in g) == 64
    assert ref_gpu.fingerprint(g) != ref_gpu.fingerprint([list(reversed(g[0]))] + g[1:])


def test_generated_kernel_matches_the_workload():
    if not ref_gpu.available(ref_gpu.DNA):
        if os.path.isdir(os.path.join(ref_gpu.REF, "bitgen")):
            assert ref_gpu.ensure_generated(ref_gpu.DNA)
        else:
            pytest.skip("neither the generated kernel nor the reference tree is here")
    meta = json.load(open(os.path.join(ref_gpu.OUT, ref_gpu.DNA + ".json")))
    assert meta["fingerprint"] == ref_gpu.fingerprint(ref_gpu.workload_groups(ref_gpu.DNA))
    src = open(os.path.join(ref_gpu.OUT, ref_gpu.DNA + ".cu")).read()
    assert 'extern "C" __global__ void KernelGenerated(' in src
    steps = ref_gpu.loop_steps(src, meta["block"])
    assert len(steps) == meta["groups"] and min(steps) >= 1
    assert "while" not in src.split("KernelGenerated")[0].split("regex_0(", 1)[-1]
