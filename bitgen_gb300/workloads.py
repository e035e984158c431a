"""Seeded synthetic pattern sets and inputs for the engine's workloads.

The public regex suites BitGen measures on (ANMLZoo / AutomataZoo, ``configs/app/full``) are not
available, so these generators stand in for them with the shapes of the five configurations the
engine is measured on:

* ``small``:      8 regexes (4-12-byte literals mixed with ``[a-z0-9]`` classes, bounded repeats
                  ``{2,5}``, one ``.*`` gap, one 2-way alternation), 4 groups, 10 KiB of printable
                  ASCII with ~20 planted matches;
* ``throughput``: 256 regexes of the same grammar, 8-40 characters, 30% with an unbounded
                  repetition (class star/plus or a ``.*`` gap), groups of 16, over 1 MiB of
                  printable ASCII tiled to 256 MiB, ~1 planted match per 4 KiB;
* ``dna``:        64 IUPAC motifs (6-20 nt, codes expanded to classes, gapped ``.{3,9}`` forms)
                  over synthetic DNA (GC 0.42, N runs of 50-5000 at rate 1e-5, LF every 80 bytes);
* ``batched``:    4096 inputs with log-normal lengths (median 8 KiB, clipped to 200 B - 64 KiB);
* ``served``:     Poisson arrivals of requests with log-uniform lengths 64 B - 4 MiB.

Every generator takes a seed and uses ``numpy.random.default_rng``.
"""

from __future__ import annotations

from dataclasses import dataclass
from typing import List, Sequence, Tuple

import numpy as np

LITERALS = "abcdefghijklmnopqrstuvwxyz0123456789"
CLASSES = [("[a-z0-9]", "abcdefghijklmnopqrstuvwxyz0123456789"), ("[0-9]", "0123456789"),
           ("[a-f]", "abcdef"), ("[aeiou]", "aeiou"), ("[a-z]", "abcdefghijklmnopqrstuvwxyz")]
PRINTABLE = bytes(range(0x20, 0x7F))


@dataclass
class PatternSet:
    regexes: List[str]
    witnesses: List[bytes]

    def groups(self, n_groups: int) -> List[List[str]]:
        from .grouping import balance_regex_groups
        return balance_regex_groups(list(self.regexes), n_groups)


def _lit(rng, k) -> str:
    return "".join(LITERALS[i] for i in rng.integers(0, len(LITERALS), size=k))


def synth_regex(rng, min_len: int, max_len: int, unbounded: str = "", alternation: bool = False) -> Tuple[str, bytes]:
    """One regex of the benchmark grammar and a string it matches.

    ``unbounded`` is "" (none), "star" (a class with ``*`` / ``+``) or "gap" (a ``.*`` gap)."""
    target = int(rng.integers(min_len, max_len + 1))
    parts: List[Tuple[str, bytes]] = []
    # a literal prefix keeps matches selective, as in real signature sets
    k = int(rng.integers(3, 6))
    s = _lit(rng, k)
    parts.append((s, s.encode()))
    special = []
    if unbounded:
        special.append(unbounded)
    if alternation:
        special.append("alt")
    cur = sum(len(p[0]) for p in parts)
    while cur < target or special:
        choice = special.pop(0) if special and (cur + 8 >= target or rng.random() < 0.3) else None
        if choice is None:
            r = rng.random()
            if r < 0.55:
                s = _lit(rng, int(rng.integers(1, 4)))
                parts.append((s, s.encode()))
            elif r < 0.8:
                cls, members = CLASSES[int(rng.integers(0, len(CLASSES)))]
                parts.append((cls, members[int(rng.integers(0, len(members)))].encode()))
            else:
                cls, members = CLASSES[int(rng.integers(0, len(CLASSES)))]
                lo = int(rng.integers(0, 3))
                hi = lo + int(rng.integers(1, 4))
                n = int(rng.integers(lo, hi + 1))
                w = "".join(members[int(rng.integers(0, len(members)))] for _ in range(n))
                parts.append((f"{cls}{{{lo},{hi}}}" if lo != hi else f"{cls}{{{lo}}}", w.encode()))
        elif choice == "star":
            cls, members = CLASSES[int(rng.integers(0, len(CLASSES)))]
            op = "*" if rng.random() < 0.5 else "+"
            n = int(rng.integers(1 if op == "+" else 0, 5))
            w = "".join(members[int(rng.integers(0, len(members)))] for _ in range(n))
            parts.append((cls + op, w.encode()))
        elif choice == "gap":
            n = int(rng.integers(0, 12))
            w = bytes(PRINTABLE[i] for i in rng.integers(0, len(PRINTABLE), size=n))
            parts.append((".*", w))
        elif choice == "alt":
            a, b = _lit(rng, int(rng.integers(2, 5))), _lit(rng, int(rng.integers(2, 5)))
            parts.append((f"({a}|{b})", (a if rng.random() < 0.5 else b).encode()))
        cur = sum(len(p[0]) for p in parts)
        if cur > max_len + 16:
            break
    # end on a literal so matches stay rare
    s = _lit(rng, 2)
    parts.append((s, s.encode()))
    return "".join(p[0] for p in parts), b"".join(p[1] for p in parts)


def pattern_set(n: int, seed: int, min_len: int, max_len: int, unbounded_frac: float,
                gap_share: float = 1 / 3, n_gap_min: int = 0, n_alt_min: int = 0) -> PatternSet:
    rng = np.random.default_rng(seed)
    regexes, wits = [], []
    kinds = []
    for i in range(n):
        if i < n_gap_min:
            kinds.append("gap")
        elif rng.random() < unbounded_frac:
            kinds.append("gap" if rng.random() < gap_share else "star")
        else:
            kinds.append("")
    for i in range(n):
        alt = i >= n_gap_min and i < n_gap_min + n_alt_min or (n_alt_min == 0 and rng.random() < 0.15)
        r, w = synth_regex(rng, min_len, max_len, kinds[i], alt)
        regexes.append(r)
        wits.append(w)
    return PatternSet(regexes, wits)


def small_patterns(seed: int = 1) -> PatternSet:
    """8 regexes: 4-12-byte literals mixed with classes and {2,5}, one .* gap, one alternation."""
    rng = np.random.default_rng(seed)
    regexes, wits = [], []
    for i in range(8):
        r, w = synth_regex(rng, 6, 16, "gap" if i == 0 else "", alternation=(i == 1))
        regexes.append(r)
        wits.append(w)
    return PatternSet(regexes, wits)


def throughput_patterns(seed: int = 3, n: int = 256) -> PatternSet:
    return pattern_set(n, seed, 8, 40, 0.30)


def printable_text(n: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return rng.integers(0x20, 0x7F, size=n, dtype=np.uint8)


def plant(text: np.ndarray, witnesses: Sequence[bytes], every: int, seed: int) -> np.ndarray:
    """Overwrite ~one witness per ``every`` bytes at seeded positions."""
    rng = np.random.default_rng(seed)
    t = text.copy()
    n = t.size
    k = max(1, n // every)
    for _ in range(k):
        w = witnesses[int(rng.integers(0, len(witnesses)))]
        if len(w) >= n:
            continue
        p = int(rng.integers(0, n - len(w)))
        t[p:p + len(w)] = np.frombuffer(w, dtype=np.uint8)
    return t


def small_workload(seed: int = 1):
    ps = small_patterns(seed)
    text = plant(printable_text(10240, seed + 1), ps.witnesses, 10240 // 20, seed + 2)
    return ps, text


def throughput_workload(total_bytes: int = 256 << 20, base_bytes: int = 1 << 20, seed: int = 3,
                        n_regex: int = 256):
    ps = throughput_patterns(seed, n_regex)
    base = plant(printable_text(base_bytes, seed + 1), ps.witnesses, 4096, seed + 2)
    reps = -(-total_bytes // base_bytes)
    return ps, base, reps


# ---------------------------------------------------------------------------------------
# DNA
# ---------------------------------------------------------------------------------------
IUPAC = {"A": "A", "C": "C", "G": "G", "T": "T", "R": "[AG]", "Y": "[CT]", "S": "[CG]",
         "W": "[AT]", "K": "[GT]", "M": "[AC]", "B": "[CGT]", "D": "[AGT]", "H": "[ACT]",
         "V": "[ACG]", "N": "[ACGT]"}


def dna_motifs(n: int = 64, seed: int = 5) -> PatternSet:
    rng = np.random.default_rng(seed)
    codes = "ACGTACGTACGTRYSWKMBDHVN"
    regexes, wits = [], []
    for i in range(n):
        L = int(rng.integers(6, 21))
        motif = "".join(codes[j] for j in rng.integers(0, len(codes), size=L))
        rx = "".join(IUPAC[c] for c in motif)
        wit = "".join(IUPAC[c].strip("[]")[int(rng.integers(0, len(IUPAC[c].strip("[]"))))] for c in motif)
        if i % 4 == 0:  # gapped form
            cut = L // 2
            lo = int(rng.integers(3, 6))
            hi = lo + int(rng.integers(2, 5))
            rx = "".join(IUPAC[c] for c in motif[:cut]) + f".{{{lo},{hi}}}" + "".join(IUPAC[c] for c in motif[cut:])
            gap = "".join("ACGT"[k] for k in rng.integers(0, 4, size=lo))
            wit = wit[:cut] + gap + wit[cut:]
        regexes.append(rx)
        wits.append(wit.encode())
    return PatternSet(regexes, wits)


def dna_text(n: int, seed: int = 6, gc: float = 0.42, line: int = 80,
             chunk: int = 64 << 20) -> np.ndarray:
    """i.i.d. A/C/G/T with the given GC fraction, runs of N (length 50-5000 at rate 1e-5 per
    byte) and a line feed after every ``line`` bytes.  Generated in chunks from 16-bit draws
    against cumulative thresholds, so a 1 GiB text needs no more than the text itself plus one
    chunk of temporaries."""
    rng = np.random.default_rng(seed)
    cum = np.cumsum([(1 - gc) / 2, gc / 2, gc / 2])
    thr = (cum * 65536).astype(np.uint32)
    seq = np.empty(n, dtype=np.uint8)
    for at in range(0, n, chunk):
        r = rng.integers(0, 65536, size=min(chunk, n - at), dtype=np.uint16)
        idx = (r >= thr[0]).astype(np.uint8)
        idx += r >= thr[1]
        idx += r >= thr[2]
        seq[at:at + r.size] = np.frombuffer(b"ACGT", dtype=np.uint8)[idx]
    n_runs = rng.poisson(n * 1e-5)
    starts = rng.integers(0, max(n, 1), size=n_runs)
    lens = rng.integers(50, 5001, size=n_runs)
    for st, ln in zip(starts.tolist(), lens.tolist()):
        seq[st:st + ln] = ord("N")
    seq[line::line + 1] = ord("\n")
    return seq


# ---------------------------------------------------------------------------------------
# batched / served
# ---------------------------------------------------------------------------------------
def batched_lengths(n: int = 4096, seed: int = 7, median: int = 8192, sigma: float = 1.0,
                    lo: int = 200, hi: int = 65536) -> np.ndarray:
    rng = np.random.default_rng(seed)
    x = np.exp(rng.normal(np.log(median), sigma, size=n))
    return np.clip(x, lo, hi).astype(np.int64)


def batched_inputs(lengths: Sequence[int], seed: int, witnesses: Sequence[bytes]) -> List[np.ndarray]:
    rng = np.random.default_rng(seed)
    out = []
    for i, n in enumerate(lengths):
        t = rng.integers(0x20, 0x7F, size=int(n), dtype=np.uint8)
        out.append(plant(t, witnesses, 4096, seed * 100003 + i))
    return out


def served_requests(n: int, seed: int = 8, lo: int = 64, hi: int = 4 << 20, rate_per_s: float = 1000.0):
    """(arrival_s, length, pattern_set_index) for n Poisson arrivals."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate_per_s, size=n)
    arrivals = np.cumsum(gaps)
    lengths = np.exp(rng.uniform(np.log(lo), np.log(hi), size=n)).astype(np.int64)
    which = rng.integers(0, 3, size=n)
    return arrivals, lengths, which
