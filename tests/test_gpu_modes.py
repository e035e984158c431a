"""GPU tests of the batched and served forms: same results as the plain form, bit for bit."""

import numpy as np
import pytest
import torch

from bitgen_gb300 import workloads
from bitgen_gb300.autotune import autotune
from bitgen_gb300.batched import BatchScanner, PerInputScanner
from bitgen_gb300.compiler import Tuning
from bitgen_gb300.engine import Program, pack_bytes
from bitgen_gb300.regex import compile_group
from bitgen_gb300.served import Request, Server, latency_stats, serve_plain
from tests.helpers import first_diff, oracle_streams

pytestmark = pytest.mark.gpu


def _patterns(n, groups, seed):
    ps = workloads.throughput_patterns(seed=seed, n=n)
    return ps, [compile_group(g) for g in ps.groups(groups)]


def test_batched_graph_equals_one_launch_per_input(cuda):
    ps, groups = _patterns(24, 3, 21)
    prog = Program(groups)
    lens = workloads.batched_lengths(400, seed=22, median=1500, lo=1, hi=20000)
    items = workloads.batched_inputs(lens, 23, ps.witnesses)
    b = BatchScanner(prog, items, graph=True)
    p = PerInputScanner(prog, items)
    for _ in range(2):          # graph replays reuse the look-back records (new epoch each time)
        b.run()
        b.sync()
    p.run()
    p.sync()
    assert torch.equal(b.counts, p.counts)
    for i in range(len(items)):
        for o in range(prog.n_outputs):
            assert torch.equal(b.stream_of(o, i), p.stream_of(o, i)), (i, o)
    for i in (0, 1, 199, 399):
        want = oracle_streams(groups, items[i])
        for o, w in enumerate(want):
            assert first_diff(b.stream_of(o, i).cpu().numpy(), w) is None


def test_served_result_alone_equals_in_the_mix(cuda):
    psA, gA = _patterns(16, 2, 31)
    psB, gB = _patterns(40, 4, 32)
    progs = {"A": Program(gA), "B": Program(gB)}
    rng = np.random.default_rng(33)
    reqs = []
    for i in range(60):
        n = int(np.exp(rng.uniform(np.log(64), np.log(200_000))))
        which = "A" if rng.random() < 0.5 else "B"
        wit = (psA if which == "A" else psB).witnesses
        data = workloads.plant(workloads.printable_text(n, 1000 + i), wit, 2048, 2000 + i)
        reqs.append(Request(i, 0.0005 * i, which, data))
    srv = Server(progs, hbm_budget=1 << 30, slots=3, max_batch_bytes=1 << 20, max_batch_inputs=16,
                 return_streams=True)
    mixed = srv.serve(reqs, realtime=True)
    plain = serve_plain(progs, reqs, realtime=False)
    assert len(mixed) == len(reqs) == len(plain)
    for r in reqs:
        prog = progs[r.pset]
        alone = prog.scan(pack_bytes([r.data]))
        assert np.array_equal(mixed[r.rid].counts, alone.counts[:, 0].cpu().numpy()), r.rid
        assert np.array_equal(plain[r.rid].counts, mixed[r.rid].counts), r.rid
        for o in range(prog.n_outputs):
            assert np.array_equal(mixed[r.rid].streams[o], alone.stream(o, 0).cpu().numpy()), (r.rid, o)
    st = latency_stats(mixed)
    assert st["p99_ms"] >= st["p50_ms"] > 0


def test_autotuner_choice_is_exact(cuda, tmp_path, monkeypatch):
    monkeypatch.setenv("BG_CACHE_DIR", str(tmp_path))
    ps, groups = _patterns(16, 2, 41)
    text = workloads.plant(workloads.printable_text(1 << 20, 42), ps.witnesses, 4096, 43)
    inp = pack_bytes([text])
    space = [Tuning(wpt=1, min_blocks=4), Tuning(wpt=2), Tuning(wpt=4, block=128, min_blocks=3)]
    best, report = autotune(groups, inp, space=space)
    assert best in space and len(report) == 3
    again, _ = autotune(groups, inp, space=space)   # cached
    assert again == best
    ref = Program(groups).scan(inp)
    got = Program(groups, tuning=best).scan(inp)
    assert torch.equal(ref.streams, got.streams) and torch.equal(ref.counts, got.counts)


def test_streamed_scans_equal_program_scan(cuda):
    """StreamScanner: five different inputs through the double-buffered copy/scan pipeline give
    the counts (and, for the last one, the streams) of Program.scan on each input."""
    from bitgen_gb300.streaming import StreamScanner
    ps = workloads.throughput_patterns(seed=3, n=64)
    prog = Program([compile_group(g) for g in ps.groups(4)])
    n = (1 << 20) + 96
    hosts = [torch.from_numpy(workloads.plant(workloads.printable_text(n, 70 + i), ps.witnesses, 300, 80 + i)).pin_memory()
             for i in range(5)]
    sc = StreamScanner(prog, n, cuda, copy_streams=3)
    handles = []
    got = []
    for h in hosts:
        handles.append(sc.submit(h))
        if len(handles) >= 2:
            got.append(sc.counts(handles[-2]))
    got.append(sc.counts(handles[-1]))
    for h, c in zip(hosts, got):
        want = prog.scan(pack_bytes([h.numpy()]))
        assert c == [int(x) for x in want.counts[:, 0].tolist()]
    last = prog.scan(pack_bytes([hosts[-1].numpy()]))
    W = last.words[0]
    assert torch.equal(sc.out[:, :W], last.streams[:, last.word_offsets[0]:last.word_offsets[0] + W])
    assert sum(got[-1]) > 0
