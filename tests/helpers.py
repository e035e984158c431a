"""Shared helpers for the parity tests: seeded inputs and oracle comparisons."""

from __future__ import annotations

import numpy as np

from oracle.pablo_ref import int_to_words, run_group, words_to_int


def rand_text(n: int, seed: int, alphabet: bytes = bytes(range(0x20, 0x7F))) -> np.ndarray:
    rng = np.random.default_rng(seed)
    a = np.frombuffer(alphabet, dtype=np.uint8)
    return a[rng.integers(0, len(a), size=n)] if n else np.zeros(0, dtype=np.uint8)


def oracle_streams(groups, data: np.ndarray, per_regex: bool = False):
    """Big-int oracle results per output, as reference-layout uint32 words."""
    W = (data.size + 31) // 32
    outs = []
    for g in groups:
        if per_regex and g.regex_results:
            res, vals = run_group(g, data, want=g.regex_results)
            outs.extend(int_to_words(vals[r], W) for r in g.regex_results)
        else:
            outs.append(int_to_words(run_group(g, data), W))
    return outs


def first_diff(a: np.ndarray, b: np.ndarray):
    a = np.asarray(a, dtype=np.uint32)
    b = np.asarray(b, dtype=np.uint32)
    if a.shape != b.shape:
        return f"shape {a.shape} vs {b.shape}"
    idx = np.nonzero(a != b)[0]
    if idx.size == 0:
        return None
    w = int(idx[0])
    return f"first mismatch at word {w} (chars {32*w}..{32*w+31}): got {a[w]:08x} want {b[w]:08x}; {idx.size} words differ"
