"""GPU: the reference-facing hooks (transpose op + kernel_0.init_kernel 5-tuple) end to end,
on the reference's quick-start known answer and on `$` / Lookahead programs."""

import importlib
import os
import sys

import numpy as np
import pytest
import torch

from bitgen_gb300.backend import byte_stream_transpose, init_kernel, write_kernel_module
from bitgen_gb300.compiler import Tuning
from bitgen_gb300.engine import Program, pack_bytes
from bitgen_gb300.grouping import group_regex_in_list
from bitgen_gb300.regex import compile_group
from oracle.pablo_ref import int_to_words, run_group
from tests.helpers import first_diff, oracle_streams, rand_text

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _reference_count(result: torch.Tensor) -> int:
    """Bitstream(result.cpu().numpy()).get_count() (bitgen/bitstream.py:27-61): popcount."""
    return int(np.unpackbits(result.cpu().numpy().view(np.uint8)).sum())


def test_readme_known_answer_through_the_drop_in_hooks(cuda, tmp_path):
    kat = np.load(os.path.join(GOLDEN, "readme_kat.npz"))
    rx = [str(r) for r in kat["regexes"]]
    groups = [compile_group(g) for g in group_regex_in_list(rx, int(kat["n_groups"]))]
    data = kat["input"]
    # bitgen/bitstream.py:166-225: pad to 32, uint8 [S=1, M=1, Npad] -> uint32 [1, 1, 8, W]
    npad = -(-data.size // 32) * 32
    bytestream = torch.zeros((1, 1, npad), dtype=torch.uint8, device=cuda)
    bytestream[0, 0, :data.size] = torch.from_numpy(data.copy())
    basis = torch.zeros((1, 1, 8, npad // 32), dtype=torch.uint32, device=cuda)
    byte_stream_transpose(bytestream, basis)
    # kernels/kernel_0.py as from_icgrep.init_kernel imports it (from_icgrep.py:169-193)
    path = write_kernel_module(groups, str(tmp_path))
    sys.path.insert(0, str(tmp_path))
    try:
        sys.modules.pop("kernels", None)
        kmod = importlib.import_module("kernels.kernel_0")
        result, tmp, handle, run_fn, dyn = kmod.init_kernel(len(groups), bytestream, basis, {})
    finally:
        sys.path.remove(str(tmp_path))
    assert tmp is None and dyn is None and tuple(result.shape) == (1, 1, len(groups), npad // 32)
    result.zero_()
    run_fn(basis)
    torch.cuda.synchronize()
    # the reference validates the popcount of all groups against icgrep's count
    assert _reference_count(result) == int(kat["expected_count"]) == 16
    # position-exact against the oracle (basis path: the zero padding is part of the input)
    for g, grp in enumerate(groups):
        want = int_to_words(run_group(grp, np.concatenate([data, np.zeros(npad - data.size, np.uint8)])),
                            npad // 32)
        assert first_diff(result[0, 0, g].cpu().numpy(), want) is None
    handle.free()
    # and with the raw-bytes path over exactly 10 000 bytes
    prog = Program(groups)
    res = prog.scan(pack_bytes([data]))
    assert int(res.counts.sum()) == 16


def test_dollar_and_lookahead_programs(cuda):
    groups = [compile_group(["ab$", "x[0-9]*$", "(cd|ef)$"]), compile_group(["^q.*z$", "k$"])]
    for wpt in (1, 2):
        prog = Program(groups, tuning=Tuning(wpt=wpt))
        assert prog.fused and prog.spec.tail_lanes >= 1
        lens = [0, 1, 2, 31, 32, 33, 63, 64, 65, 1000, 5000, 40000]
        items = [rand_text(n, 77 + n, b"abcdefxz09kq\n") for n in lens]
        inp = pack_bytes(items)
        res = prog.scan(inp)
        for i, data in enumerate(items):
            want = oracle_streams(groups, data)
            for o, w in enumerate(want):
                assert first_diff(res.stream(o, i).cpu().numpy(), w) is None, (wpt, i, o)
    interp = Program(groups, executor="interp")
    r2 = interp.scan(pack_bytes(items))
    for i in range(len(items)):      # padding words between inputs are not part of any output
        for o in range(prog.n_outputs):
            assert torch.equal(r2.stream(o, i), res.stream(o, i)), (i, o)
    assert torch.equal(r2.counts, res.counts)
