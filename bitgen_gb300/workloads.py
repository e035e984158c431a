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
CLASS = "[a-z0-9]"                  # the grammar's bracket class; its members are LITERALS
PRINTABLE = bytes(range(0x20, 0x7F))
LIT_MIN, LIT_MAX = 4, 12            # literal length
REP_LO, REP_HI = 2, 5               # the bounded repeat {2,5}


@dataclass
class PatternSet:
    regexes: List[str]
    witnesses: List[bytes]

    def groups(self, n_groups: int) -> List[List[str]]:
        from .grouping import balance_regex_groups
        return balance_regex_groups(list(self.regexes), n_groups)


def _lit(rng, k) -> str:
    return "".join(LITERALS[i] for i in rng.integers(0, len(LITERALS), size=k))


def _members(rng, k) -> bytes:
    return _lit(rng, k).encode()


def synth_regex(rng, min_len: int, max_len: int, unbounded: str = "", alternation: bool = False) -> Tuple[str, bytes]:
    """One regex of the benchmark grammar and a string it matches.

    A regex is literals of 4-12 bytes over [a-z0-9] separated by class pieces, starting and
    ending with a literal; a class piece is ``[a-z0-9]`` or the bounded repeat
    ``[a-z0-9]{2,5}``.  The regex text is min_len..max_len characters long (a single literal
    when the length leaves no room for a class piece).  ``unbounded`` turns one class piece
    into an unbounded repetition: "star" gives ``[a-z0-9]*`` or ``[a-z0-9]+`` (MatchStar),
    "gap" a ``.*`` gap.  ``alternation`` turns one literal after the first into a two-way
    alternation of 4-6-byte literals."""
    target = int(rng.integers(min_len, max_len + 1))
    parts: List[Tuple[str, bytes]] = []

    def literal(room: int) -> Tuple[str, bytes]:
        k = int(rng.integers(LIT_MIN, LIT_MAX + 1))
        k = max(LIT_MIN, min(k, room))
        s = _lit(rng, k)
        return s, s.encode()

    special = []
    if unbounded:
        special.append(unbounded)
    if alternation:
        special.append("alt")
    cur = 0
    parts.append(literal(min(LIT_MAX, target if (special or target < 16) else target - 12)))
    cur = len(parts[0][0])
    while cur < target or special:
        # the class piece: a pending unbounded repetition, else [a-z0-9] or [a-z0-9]{2,5}
        if special and special[0] in ("star", "gap") and (target - cur < 30 or rng.random() < 0.6):
            kind = special.pop(0)
            if kind == "star":
                op = "*" if rng.random() < 0.5 else "+"
                n = int(rng.integers(1 if op == "+" else 0, 5))
                sep = (CLASS + op, _members(rng, n))
            else:
                n = int(rng.integers(0, 12))
                sep = (".*", bytes(PRINTABLE[i] for i in rng.integers(0, len(PRINTABLE), size=n)))
        elif rng.random() < 0.5:
            sep = (CLASS, _members(rng, 1))
        else:
            sep = (f"{CLASS}{{{REP_LO},{REP_HI}}}", _members(rng, int(rng.integers(REP_LO, REP_HI + 1))))
        if not special and cur + len(sep[0]) + LIT_MIN > max_len:
            break
        parts.append(sep)
        cur += len(sep[0])
        if special and special[0] == "alt" and (target - cur < 16 or rng.random() < 0.5):
            special.pop(0)
            a = _lit(rng, int(rng.integers(LIT_MIN, 7)))
            b = _lit(rng, int(rng.integers(LIT_MIN, 7)))
            parts.append((f"({a}|{b})", (a if rng.random() < 0.5 else b).encode()))
        else:
            parts.append(literal(max(LIT_MIN, min(target, max_len) - cur)))
        cur += len(parts[-1][0])
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
        r, w = synth_regex(rng, 8, 24, "gap" if i == 0 else "", alternation=(i == 1))
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
