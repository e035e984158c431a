"""CPU: the seeded synthetic workloads have the shapes and value distributions they stand in for
(the public regex suites and inputs BitGen measures on are absent): pattern-set sizes and
lengths, the share of unbounded repetitions, the text alphabets and line structure, planted
matches that the regexes really match, and the batched / served length and arrival laws."""

import re

import numpy as np

from bitgen_gb300 import workloads
from oracle.nfa_ref import match_ends


def test_small_workload():
    ps, text = workloads.small_workload()
    assert len(ps.regexes) == 8 and text.size == 10240
    assert text.min() >= 0x20 and text.max() <= 0x7E
    assert any(".*" in r for r in ps.regexes) and any("|" in r for r in ps.regexes)
    data = text.tobytes()
    ends = sum(bin(match_ends(r, data)).count("1") for r in ps.regexes)
    assert ends >= 10                                     # the planted witnesses match


def test_throughput_pattern_set():
    ps = workloads.throughput_patterns(seed=3, n=256)
    assert len(ps.regexes) == len(ps.witnesses) == 256
    unbounded = [r for r in ps.regexes if re.search(r"\*|\+", r)]
    assert 0.2 <= len(unbounded) / 256 <= 0.4            # about 30%
    for r, w in zip(ps.regexes[:64], ps.witnesses[:64]):
        assert match_ends(r, w) >> (len(w) - 1) & 1, r   # every witness ends a match of its regex
    ps2, base, reps = workloads.throughput_workload(total_bytes=8 << 20, base_bytes=1 << 20)
    assert base.size == 1 << 20 and reps == 8
    assert base.min() >= 0x20 and base.max() <= 0x7E and not np.any(base == 0x0A)   # no LF


def test_dna_text_and_motifs():
    ps = workloads.dna_motifs(64, seed=5)
    assert len(ps.regexes) == 64
    assert sum(1 for r in ps.regexes if re.search(r"\.\{\d+,\d+\}", r)) == 16   # every 4th gapped
    text = workloads.dna_text(1 << 20, seed=6)
    assert np.all(text[79::81] == 0x0A) or np.all(text[80::81] == 0x0A)
    body = text[text != 0x0A]
    assert set(np.unique(body).tolist()) <= set(b"ACGTN")
    acgt = body[body != ord("N")]
    gc = np.isin(acgt, np.frombuffer(b"GC", np.uint8)).mean()
    assert abs(gc - 0.42) < 0.01


def test_batched_and_served_laws():
    lens = workloads.batched_lengths(4096, seed=7)
    assert lens.min() >= 200 and lens.max() <= 65536
    assert abs(np.median(lens) / 8192 - 1) < 0.1
    arr, rl, which = workloads.served_requests(20000, seed=8, rate_per_s=500.0)
    assert np.all(np.diff(arr) >= 0)
    assert abs(np.mean(np.diff(arr)) * 500.0 - 1) < 0.05          # Poisson at the given rate
    assert rl.min() >= 64 and rl.max() <= 4 << 20
    logs = np.log(rl)
    assert abs(np.mean(logs) - (np.log(64) + np.log(4 << 20)) / 2) < 0.1   # log-uniform
    assert set(np.unique(which).tolist()) == {0, 1, 2}
