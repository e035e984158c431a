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
    assert check_grammar(ps, 8, 40) == 1.0 and any("{2,5}" in r for r in ps.regexes)
    data = text.tobytes()
    ends = sum(bin(match_ends(r, data)).count("1") for r in ps.regexes)
    assert ends >= 10                                     # the planted witnesses match


PIECE = re.compile(r"\[a-z0-9\](\{2,5\}|\*|\+)?|\.\*|\(([a-z0-9]+)\|([a-z0-9]+)\)|([a-z0-9]+)")


def grammar_pieces(rx: str):
    """The pieces of a regex of the benchmark grammar; fails on anything else."""
    out, at = [], 0
    while at < len(rx):
        m = PIECE.match(rx, at)
        assert m, f"{rx!r}: no grammar piece at {at}"
        out.append(m)
        at = m.end()
    return out


def check_grammar(ps, lo: int, hi: int):
    """4-12-byte literals over [a-z0-9], [a-z0-9] classes with the bounded repeat {2,5} or an
    unbounded repetition, .* gaps, two-way alternations; regex text lo..hi characters."""
    within = 0
    for rx in ps.regexes:
        pieces = grammar_pieces(rx)
        assert pieces[0].group(4), f"{rx!r} starts with a literal"
        for m in pieces:
            if m.group(4):
                assert 4 <= len(m.group(4)) <= 12, rx
            if m.group(2):
                assert 4 <= len(m.group(2)) <= 6 and 4 <= len(m.group(3)) <= 6, rx
        within += lo <= len(rx) <= hi
    return within / len(ps.regexes)


def test_throughput_pattern_set():
    ps = workloads.throughput_patterns(seed=3, n=256)
    assert len(ps.regexes) == len(ps.witnesses) == 256
    assert check_grammar(ps, 8, 40) >= 0.95
    assert any("{2,5}" in r for r in ps.regexes) and any(".*" in r for r in ps.regexes)
    assert any("|" in r for r in ps.regexes)
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
