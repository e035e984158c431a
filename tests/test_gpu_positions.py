"""Positions-only scans: a program whose parts share outputs, launched without output streams,
must count every set bit once and list exactly the positions the dense scan sets.

Two regexes of one group that end at the same positions (one a suffix of the other) sit in
different parts, so their bits collide in one output; the position set must count them once.
Compared with the dense scan (bg_plan_launch with output streams) and with the oracle."""

import numpy as np
import pytest
import torch

from bitgen_gb300 import _native as N
from bitgen_gb300 import workloads
from bitgen_gb300.engine import Program, bytes_input
from bitgen_gb300.regex import compile_group
from tests.helpers import oracle_streams


def _positions_from_streams(streams: np.ndarray, n: int):
    """Sorted (output << 52 | position) keys of the set bits of dense streams [n_out][W]."""
    keys = []
    for o, s in enumerate(streams):
        bits = np.unpackbits(s.astype(">u4").view(np.uint8))
        pos = np.nonzero(bits[:n])[0].astype(np.uint64)
        keys.append((np.uint64(o) << np.uint64(52)) | pos)
    return np.sort(np.concatenate(keys)) if keys else np.zeros(0, np.uint64)


@pytest.fixture(scope="module")
def colliding(cuda):
    ps = workloads.throughput_patterns(seed=21, n=60)
    groups = ps.groups(4)
    wits = list(ps.witnesses)
    # suffix pairs, each kept in one group (one output): every match of the first regex ends
    # a match of the second at the same position
    for g, a in zip(groups, ("q7k2m9x4z", "b8v3n6w1c")):
        g += [a, a[4:]]
        wits.append(a.encode())
    prog = Program([compile_group(g) for g in groups])
    assert prog.fused and prog.merges and prog.spec.n_parts > 1
    return prog, groups, wits


def _text(n, wits, seed):
    return workloads.plant(workloads.printable_text(n, seed), wits, 1500, seed + 1)


@pytest.mark.gpu
@pytest.mark.parametrize("n", [70_001, 3_000_000])
def test_positions_only_equals_dense(colliding, cuda, n):
    prog, groups, wits = colliding
    text = _text(n, wits, 30)
    data = torch.from_numpy(text).to(cuda)
    dense = prog.scan(bytes_input(data), positions=True)
    sparse = prog.scan(bytes_input(data), streams=False, positions=True, pos_capacity=1 << 16)
    assert sparse.streams is None
    W = -(-n // 32)
    got_dense = dense.streams[:, :W].cpu().numpy().view(np.uint32)
    want_keys = _positions_from_streams(got_dense, n)
    assert want_keys.size > n // 4000
    # both the dense launch's positions and the positions-only launch's equal the streams' bits
    assert np.array_equal(np.sort(dense.positions), want_keys)
    assert np.array_equal(sparse.positions, want_keys), "positions-only launch differs"
    assert torch.equal(sparse.counts, dense.counts)
    # the colliding pairs really collide: their regexes' ends coincide in outputs 0 and 1
    assert int(dense.counts[0, 0]) > 0 and int(dense.counts[1, 0]) > 0
    if n <= 100_000:
        want = oracle_streams([compile_group(g) for g in groups], text)
        for o, w in enumerate(want):
            assert np.array_equal(got_dense[o], w), o
            assert int(sparse.counts[o, 0]) == int(np.unpackbits(w.view(np.uint8)).sum())


@pytest.mark.gpu
def test_counts_only_through_the_position_set(colliding, cuda):
    prog, _, wits = colliding
    text = _text(1_000_000, wits, 31)
    data = torch.from_numpy(text).to(cuda)
    inp = bytes_input(data)
    dense = prog.scan(inp)
    plan = prog.plan(inp, dense.word_offsets, dense.streams.shape[1])
    plan.set_positions(None, count_capacity=1 << 15)
    counts = torch.empty_like(dense.counts)
    sp = int(torch.cuda.current_stream().cuda_stream)
    plan.launch(data.data_ptr(), 0, counts.data_ptr(), sp)
    plan.sync(sp)
    plan.set_positions(None)
    assert torch.equal(counts, dense.counts)


@pytest.mark.gpu
def test_position_set_overflow_is_reported(colliding, cuda):
    """More distinct positions than twice the capacity: BG_ERR_CAPACITY, no fault; the next
    launch with room is exact again."""
    prog, _, wits = colliding
    text = _text(4_000_000, wits, 32)
    data = torch.from_numpy(text).to(cuda)
    dense = prog.scan(bytes_input(data))
    total = int(dense.counts.sum())
    assert total > 1024 + 200          # the smallest set has 1024 slots
    with pytest.raises(RuntimeError, match="capacity|incomplete"):
        prog.scan(bytes_input(data), streams=False, positions=True, pos_capacity=100)
    again = prog.scan(bytes_input(data), streams=False, positions=True, pos_capacity=1 << 16)
    assert torch.equal(again.counts, dense.counts)
