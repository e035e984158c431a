"""The allocation-free scan (bg_scan_noalloc) against the plan path (bg_plan_launch).

bg_scan_noalloc keeps its look-back records, tables and state in one fixed device array of the
library.  These tests call it through the C ABI and require bit-exact agreement with the plan
path.  That holds on two calls in a row, which share the array, on the largest input the array
admits and on an empty input.  Free device memory must not move across a call, and one byte
past the limit must be rejected.  The file is named so that pytest collects it last: it must
pass alone in a fresh process and after every other test.
"""

import ctypes as C
import os
import re

import numpy as np
import pytest
import torch

from bitgen_gb300 import _native as N
from bitgen_gb300 import workloads
from bitgen_gb300.engine import Program, bytes_input

HEADER = os.path.join(os.path.dirname(os.path.dirname(__file__)), "include", "bitgen_gb300.h")
SCRATCH_BYTES = 4 << 20
RECORDS = SCRATCH_BYTES // 8 - 32


def test_header_states_the_limit_and_bad_arguments_fail(native):
    txt = open(HEADER).read()
    assert re.search(r"#define BG_NOALLOC_SCRATCH_BYTES \(4u << 20\)", txt)
    assert "BG_NOALLOC_SCRATCH_BYTES / 8u - 32u" in txt
    # argument checks come before any device work, so they run without a GPU
    assert native.bg_scan_noalloc(None, None, 0, None, 0, None, None, None) == N.BG_ERR_INVALID
    assert b"bg_scan_noalloc" in native.bg_last_error()


def _noalloc(prog: Program, data: torch.Tensor, n: int, out, counts, status, stream=None):
    return N.lib().bg_scan_noalloc(
        prog._handle, data.data_ptr(), n, out.data_ptr() if out is not None else None,
        out.shape[1] if out is not None else 0, counts.data_ptr() if counts is not None else None,
        status.data_ptr(), stream)


def _plan_path(prog: Program, data: torch.Tensor, n: int):
    """Streams [n_outputs][W] and counts [n_outputs] from the plan path (bg_plan_launch)."""
    res = prog.scan(bytes_input(data[:n]))
    W = -(-n // 32)
    o = res.word_offsets[0]
    return res.streams[:, o:o + W].cpu().numpy(), res.counts[:, 0].cpu().numpy()


@pytest.fixture(scope="module")
def program(cuda):
    ps = workloads.throughput_patterns(seed=11, n=48)
    prog = Program.from_regex_groups(ps.groups(4))
    assert prog.fused
    return prog, ps


def _text(n, ps, seed):
    return workloads.plant(workloads.printable_text(n, seed), ps.witnesses, 2048, seed + 1)


@pytest.mark.gpu
def test_two_calls_in_a_row_match_the_plan_path(program, cuda):
    prog, ps = program
    sizes = (3_000_001, 1_234_567)
    datas = [torch.from_numpy(_text(n, ps, 20 + i)).to(cuda) for i, n in enumerate(sizes)]
    want = [_plan_path(prog, d, n) for d, n in zip(datas, sizes)]
    W = [-(-n // 32) for n in sizes]
    outs = [torch.full((prog.n_outputs, w + 3), 0x5A5A5A5A, dtype=torch.int32, device=cuda) for w in W]
    cnts = [torch.full((prog.n_outputs,), -1, dtype=torch.int64, device=cuda) for _ in sizes]
    stats = [torch.full((1,), -1, dtype=torch.int32, device=cuda) for _ in sizes]
    torch.cuda.synchronize()
    for i, n in enumerate(sizes):   # back to back on the default stream, no sync in between
        assert _noalloc(prog, datas[i], n, outs[i], cnts[i], stats[i]) == N.BG_OK, N.lib().bg_last_error()
    torch.cuda.synchronize()
    for i, n in enumerate(sizes):
        assert int(stats[i].item()) == 0
        got = outs[i].cpu().numpy().view(np.uint32)
        ws, wc = want[i]
        assert np.array_equal(got[:, :W[i]], ws), i
        assert np.all(got[:, W[i]:] == 0x5A5A5A5A), "wrote past the input's words"
        assert np.array_equal(cnts[i].cpu().numpy(), wc), i
        assert wc.sum() > 0
    # a call after the first one on this device allocates nothing
    again = torch.full((1,), -1, dtype=torch.int32, device=cuda)
    torch.cuda.synchronize()
    before = torch.cuda.mem_get_info()[0]
    assert _noalloc(prog, datas[0], sizes[0], outs[0], cnts[0], again) == N.BG_OK
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == before
    assert int(again.item()) == 0
    assert np.array_equal(outs[0].cpu().numpy().view(np.uint32)[:, :W[0]], want[0][0])


@pytest.mark.gpu
def test_limit_is_exact_and_enforced(program, cuda):
    prog, ps = program
    tile_words = prog.spec.tile_words
    s = prog.spec

    def words(tiles):   # the scratch rule stated in include/bitgen_gb300.h
        rows = -(-tiles // 32)
        w = s.n_parts * (rows + 1) + 512 + s.n_run * rows if s.n_run else 0
        return (max(1, s.n_adds) * tiles + (3 * s.n_pre * rows + 1) // 2
                + (s.n_run * tiles + 1) // 2 + (w + 1) // 2)
    lo, hi = 1, RECORDS
    while hi - lo > 1:
        mid = (lo + hi) // 2
        lo, hi = (mid, hi) if words(mid) <= RECORDS else (lo, mid)
    max_tiles = lo
    n_max = max_tiles * tile_words * 32
    data = torch.from_numpy(_text(n_max + 32, ps, 40)).to(cuda)
    out = torch.empty((prog.n_outputs, n_max // 32 + 1), dtype=torch.int32, device=cuda)
    cnt = torch.empty((prog.n_outputs,), dtype=torch.int64, device=cuda)
    st = torch.full((1,), -1, dtype=torch.int32, device=cuda)
    # the largest input the fixed scratch admits is accepted and exact
    assert _noalloc(prog, data, n_max, out, cnt, st) == N.BG_OK, N.lib().bg_last_error()
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    ws, wc = _plan_path(prog, data, n_max)
    assert np.array_equal(out.cpu().numpy().view(np.uint32)[:, :n_max // 32], ws)
    assert np.array_equal(cnt.cpu().numpy(), wc)
    # one byte more needs one more tile and is rejected before anything is enqueued
    assert _noalloc(prog, data, n_max + 1, out, cnt, st) == N.BG_ERR_CAPACITY
    msg = N.lib().bg_last_error().decode()
    assert "scratch" in msg and str(n_max) in msg
    # an output row shorter than the input is rejected too
    assert _noalloc(prog, data, n_max, out[:, :8], cnt, st) == N.BG_ERR_INVALID


def _max_bytes(prog: Program) -> int:
    """Largest input (whole tiles) the fixed scratch admits for this program."""
    s = prog.spec

    def words(tiles):   # the scratch rule stated in include/bitgen_gb300.h
        rows = -(-tiles // 32)
        w = s.n_parts * (rows + 1) + 512 + s.n_run * rows if s.n_run else 0
        return (max(1, s.n_adds) * tiles + (3 * s.n_pre * rows + 1) // 2
                + (s.n_run * tiles + 1) // 2 + (w + 1) // 2)
    lo, hi = 1, RECORDS
    while hi - lo > 1:
        mid = (lo + hi) // 2
        lo, hi = (mid, hi) if words(mid) <= RECORDS else (lo, mid)
    return lo * s.tile_words * 32


@pytest.mark.gpu
def test_record_range_moves_over_an_earlier_calls_masks(program, cuda):
    """A call whose look-back records reach past the previous call's records lands on words
    that call used as run masks and work list (untagged values).  Programs and sizes alternate
    so that the record range grows and shrinks; every call must equal the plan path."""
    prog_a, ps_a = program
    ps_b = workloads.pattern_set(40, seed=12, min_len=8, max_len=40, unbounded_frac=0.9)
    prog_b = Program.from_regex_groups(ps_b.groups(4))
    assert prog_a.spec.n_run > 0 and prog_b.spec.n_run > 0
    assert prog_b.spec.n_adds > prog_a.spec.n_adds
    cases = []
    for prog, ps, frac, seed in ((prog_a, ps_a, 1.0, 50), (prog_b, ps_b, 1.0, 51),
                                 (prog_a, ps_a, 0.5, 52), (prog_b, ps_b, 0.9, 53),
                                 (prog_a, ps_a, 1.0, 54)):
        n = max(32, int(_max_bytes(prog) * frac) // 32 * 32 - 32)
        data = torch.from_numpy(_text(n, ps, seed)).to(cuda)
        cases.append((prog, data, n, _plan_path(prog, data, n)))
    outs = [torch.empty((p.n_outputs, -(-n // 32)), dtype=torch.int32, device=cuda)
            for p, _, n, _ in cases]
    cnts = [torch.empty((p.n_outputs,), dtype=torch.int64, device=cuda) for p, _, _, _ in cases]
    stats = [torch.full((1,), -1, dtype=torch.int32, device=cuda) for _ in cases]
    torch.cuda.synchronize()
    for i, (prog, data, n, _) in enumerate(cases):   # back to back, one stream
        assert _noalloc(prog, data, n, outs[i], cnts[i], stats[i]) == N.BG_OK, N.lib().bg_last_error()
    torch.cuda.synchronize()
    for i, (prog, data, n, (ws, wc)) in enumerate(cases):
        assert int(stats[i].item()) == 0, i
        assert np.array_equal(outs[i].cpu().numpy().view(np.uint32), ws), i
        assert np.array_equal(cnts[i].cpu().numpy(), wc), i
    prog_b.close()


@pytest.mark.gpu
def test_empty_input(program, cuda):
    prog, _ = program
    data = torch.zeros(32, dtype=torch.uint8, device=cuda)
    out = torch.zeros((prog.n_outputs, 4), dtype=torch.int32, device=cuda)
    cnt = torch.full((prog.n_outputs,), -1, dtype=torch.int64, device=cuda)
    st = torch.full((1,), -1, dtype=torch.int32, device=cuda)
    assert _noalloc(prog, data, 0, out, cnt, st) == N.BG_OK
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    assert np.all(cnt.cpu().numpy() == 0)
