"""Q-gram prefilter: which terms of a program can be non-zero in a tile, decided from the
tile's bytes before any bitstream is computed.

Position bounds.  PB[v][k] is the set of byte values that can stand k positions before a set
bit of node v (``position_bounds``: AND intersects, OR / XOR / SEL unite, Advance shifts, a
class bounds its own position).  A *window* of node z is a run of W = q + s - 1 consecutive
positions k = o .. o + W - 1 whose bounds are all constrained: when z is set at p, the bytes
p - o - W + 1 .. p - o lie in those sets, so one of the s q-grams of the window (ending at
p - o - j, j < s) ends at a position that is a multiple of s plus s - 1.  The kernel probes
exactly those q-grams: with stride s it looks at one q-gram in s positions.  When none of
the window's q-grams occurs among the warp's bytes, z is zero in all of the warp's exact
lanes (the window lies inside the bytes the warp computes, since it is no deeper than the
program's halo).

Configurations (q, s): (4, 2) probes 16 four-byte q-grams per 32 bytes and needs windows of
five positions (a literal of five bytes, or four bytes and a small class); (4, 1) and (3, 1)
need four and three.  ``build`` picks, per program, the configuration with the lowest
estimated cost per tile: probes, expected Bloom hits (each resolved on the slow path) and
terms run.

Zero implication.  Z(v) is the set of window nodes whose being zero makes v zero: AND and
Advance / Lookahead inherit the union of their operands' sets, OR / XOR / SEL the intersection,
and an addition its marker's set.  The last rule holds only while no carry enters the tile, so
the kernel also runs a term whenever one of its additions could take or owe a carry: a
look-back addition whose class is all ones at its carry lane or at its successor's, or a
pre-pass addition with a carry-in when the term's filter holds only through it.

Each term (an OR-ed leaf of an output) gets the most selective window of Z(term) as its
filter, preferring one that does not pass through a pre-pass addition; a term without one
always runs.  Each pre-pass addition gets the filter of its marker, so the pre-pass can skip
the marker's computation too.

Extensions.  Where the bounds also fix single bytes 1, 2 and 3 positions before a q-gram, the
table holds, under the q-gram, an extension record (those bytes and the term's bit), and the
kernel sets the bit only when the bytes before the q-gram match.

Wildcards.  A 4-gram may leave its oldest or its newest byte unconstrained (a literal of four
bytes probed at stride 2 has, in one phase, only three known bytes in the probed gram).  Its
Bloom bits are set for all 256 values of that byte; the exact table holds it once, with the
byte zeroed, and a Bloom hit is looked up as itself and with that byte zeroed.  Sharing the
table with exact keys can only add bits (a masked lookup that finds an exact key whose byte is
zero), never lose one.

The kernel probes the q-grams in a Bloom bitmap (2^20 bits by default, in shared memory) and
resolves the rare hits in an exact open-addressed table that maps a q-gram to the records of
the filters containing it.  Both tables are generated here and compiled into the kernel.
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Dict, FrozenSet, List, Optional, Sequence, Tuple

ALL = (1 << 256) - 1
WILD_OLD, WILD_NEW = 1, 2   # a 4-gram whose oldest / newest byte is unconstrained
MAX_KEYS = 4096         # most q-grams one filter may register
MAX_EXT = 3             # bytes before a q-gram an extension record may fix
DEPTH = 12              # positions before a set bit the bounds are followed for
BLOOM_BITS = 20         # log2 of the Bloom bitmap size (128 KB of shared memory)
HASH_BLOOM = 0x9E3779B1
HASH_EXACT = 0x85EBCA6B
CONFIGS = ((4, 2), (4, 1), (3, 1))   # (q, stride), cheapest probes first
# estimated warp instructions per tile, for choosing the configuration: a probe per lane, a
# Bloom hit (recorded, then looked up with up to 31 others of its chunk at once), a term run
# by the execute pass.  On the 256-regex workload stride 2 (1.6 hits per tile) measured 3%
# faster over the whole scan than stride 1 (0.5 hits per tile)
COST_PROBE, COST_HIT, COST_RUN = 5.0, 40.0, 600.0


def bloom_hash(key: int, bits: int = BLOOM_BITS, q: int = 3) -> int:
    """Bit index of q-gram `key` (oldest byte in bits 0-7) in a 2^bits-bit Bloom bitmap, as the
    kernel computes it (bg_device.cuh bloom_probe): the word is the top bits - 5 bits of the
    32-bit product key * HASH_BLOOM (of the 24-bit product shifted up by 8 for a trigram, so
    that the byte above it does not matter), the bit within the word is the key's low 5 bits."""
    if q == 3:
        h = ((key & 0xFFFFFF) * HASH_BLOOM << 8) & 0xFFFFFFFF
    else:
        h = (key * HASH_BLOOM) & 0xFFFFFFFF
    return ((h >> (32 - bits + 5)) << 5) | (key & 31)


def exact_hash(key: int, log2_slots: int) -> int:
    return ((key * HASH_EXACT) & 0xFFFFFFFF) >> (32 - log2_slots)


def _bytes(s: int) -> List[int]:
    return [b for b in range(256) if (s >> b) & 1]


def _n(s: int) -> int:
    return bin(s).count("1")


def position_bounds(gen, depth: int = DEPTH) -> Dict[int, Tuple[int, ...]]:
    """PB[v][k]: set of byte values that can stand k positions before a set bit of node v
    (k < depth; ALL when unconstrained).  AND intersects its operands' bounds, OR / XOR / SEL
    unite them, Advance(a, s) moves a's bounds s positions back, a class bounds its own position
    only; additions, NOT of a heavy node and Lookahead bound nothing."""
    d = gen.d
    PB: Dict[int, Tuple[int, ...]] = {}
    free = (ALL,) * depth
    for v in sorted(gen.live):
        n = d.nodes[v]
        if d.is_cc(v):
            PB[v] = (gen.byteset(v),) + (ALL,) * (depth - 1)
        elif n.op == "and":
            a, b = PB[n.args[0]], PB[n.args[1]]
            PB[v] = tuple(x & y for x, y in zip(a, b))
        elif n.op in ("or", "xor"):
            a, b = PB[n.args[0]], PB[n.args[1]]
            PB[v] = tuple(x | y for x, y in zip(a, b))
        elif n.op == "sel":
            a, b = PB[n.args[1]], PB[n.args[2]]
            PB[v] = tuple(x | y for x, y in zip(a, b))
        elif n.op == "advance":
            a, sft = PB[n.args[0]], n.shift
            PB[v] = tuple(a[k - sft] if k >= sft else ALL for k in range(depth))
        elif n.op == "zero":
            PB[v] = (0,) * depth
        else:
            PB[v] = free
    return PB


@dataclass(frozen=True)
class Window:
    """q-grams of one filter: grams[j] = byte sets of the q-gram ending j positions before the
    window's end (oldest byte first), ext[j] = single bytes fixed before it (nearest first)."""
    grams: Tuple[Tuple[int, ...], ...]
    ext: Tuple[Tuple[int, ...], ...]

    def keys(self) -> int:
        """Bloom keys (a wildcard byte counts 256)."""
        return sum(math.prod(_n(x) for x in g) for g in self.grams)

    def chance(self, alpha: int) -> float:
        """Expected table hits per probe on text uniform over `alpha` (before extensions)."""
        na = max(1, _n(alpha))
        return sum(math.prod(_n(x & alpha) / na for x in g) for g in self.grams)

    def exact_chance(self, alpha: int) -> float:
        na = max(1, _n(alpha))
        return sum(math.prod(_n(x & alpha) / na for x in g) * (1.0 / na) ** len(e)
                   for g, e in zip(self.grams, self.ext))


def windows(gen, PB, q: int, stride: int) -> Dict[int, List[Window]]:
    """Every window of every heavy live node for q-grams probed at `stride`."""
    d = gen.d
    W = q + stride - 1
    out: Dict[int, List[Window]] = {}
    for z in sorted(gen.live):
        if d.is_cc(z):
            continue
        b = PB[z]
        ws = []
        for o in range(0, len(b) - W + 1):
            seg = b[o:o + W]
            if any(x == 0 for x in seg):
                continue
            grams, exts = [], []
            for j in range(stride):
                # the q-gram ending at distance o + j covers distances o + j .. o + j + q - 1
                g = tuple(b[o + j + q - 1 - i] for i in range(q))      # oldest first
                if wildcard(g) < 0:
                    break
                e = []
                for k in range(o + j + q, min(len(b), o + j + q + MAX_EXT)):
                    if _n(b[k]) != 1:
                        break
                    e.append(b[k].bit_length() - 1)
                grams.append(g)
                exts.append(tuple(e))
            if len(grams) < stride:
                continue
            w = Window(tuple(grams), tuple(exts))
            if w.keys() <= MAX_KEYS:
                ws.append(w)
        if ws:
            out[z] = ws
    return out


def zero_sets(gen, tri, blocked=frozenset()) -> Dict[int, FrozenSet[int]]:
    """Z(v) for every live node (`tri`: the nodes that have a window).  The result of an
    addition in `blocked` implies nothing (its carry may be non-zero whatever its marker)."""
    d = gen.d
    Z: Dict[int, FrozenSet[int]] = {}
    empty: FrozenSet[int] = frozenset()
    for v in sorted(gen.live):
        n = d.nodes[v]
        if d.is_cc(v) or n.op in ("basis", "zero", "ones", "not"):
            z = empty
        elif n.op == "and":
            z = Z[n.args[0]] | Z[n.args[1]]
        elif n.op in ("advance", "lookahead"):
            z = Z[n.args[0]]
        elif n.op in ("or", "xor"):
            z = Z[n.args[0]] & Z[n.args[1]]
        elif n.op == "sel":
            z = Z[n.args[1]] & Z[n.args[2]]
        elif n.op in ("matchstar", "scanthru"):
            z = empty if v in blocked else Z[n.args[0]]
        else:
            z = empty
        if v in tri:
            z = z | {v}
        Z[v] = z
    return Z


def qgram_set(sets: Tuple[int, ...]) -> List[int]:
    """Keys of a q-gram with these byte sets (oldest first): oldest byte in bits 0-7."""
    keys = [0]
    for i, s in enumerate(sets):
        keys = [k | (b << (8 * i)) for k in keys for b in _bytes(s)]
    return keys


def wildcard(g: Tuple[int, ...]) -> int:
    """0 for a gram of constrained bytes; WILD_OLD / WILD_NEW when only its oldest / newest
    byte is unconstrained (4-grams only); -1 for any other gram with an unconstrained byte."""
    free = [i for i, x in enumerate(g) if x == ALL]
    if not free:
        return 0
    if len(g) == 4 and free == [0]:
        return WILD_OLD
    if len(g) == 4 and free == [len(g) - 1]:
        return WILD_NEW
    return -1


def table_keys(g: Tuple[int, ...]) -> List[int]:
    """Exact-table keys of a gram: a wildcard byte is stored as zero."""
    return qgram_set(tuple(1 if x == ALL else x for x in g))


@dataclass
class TermFilter:
    """Per-program prefilter: bit r (r < n_terms) = term r may be non-zero, bit n_terms + k =
    pre-pass addition k's marker may be non-zero.  ``always`` holds the terms without a filter.
    q-grams of q bytes are probed at the positions that are a multiple of ``stride`` plus
    stride - 1 (of a 32-byte aligned lane)."""
    n_terms: int
    n_pre: int
    term_node: List[Optional[int]]
    pre_node: List[Optional[int]]
    term_cond: List[bool] = field(default_factory=list)  # filter implies zero only if no carry
    table: Dict[int, int] = field(default_factory=dict)   # q-gram -> bits it sets by itself
    # q-gram -> extension records (bytes 1, 2, 3 positions before it packed nearest first in
    # bits 0-7, 8-15, 16-23, their number, bit): the bit is set when those bytes precede it
    ext: Dict[int, List[Tuple[int, int, int]]] = field(default_factory=dict)
    q: int = 3
    stride: int = 1
    alphabet: int = 0                                     # estimated text alphabet (bit set)
    windows: List[Optional[Window]] = field(default_factory=list)
    wild_old: FrozenSet[int] = frozenset()   # table keys of grams with a free oldest byte
    wild_new: FrozenSet[int] = frozenset()   # ... with a free newest byte
    cost: float = 0.0                                     # estimated instructions per tile
    hits: float = 0.0                                     # estimated slow-path hits per tile

    @property
    def n_bits(self) -> int:
        return self.n_terms + self.n_pre

    @property
    def words(self) -> int:
        return max(1, (self.n_bits + 31) // 32)

    @property
    def enabled(self) -> bool:
        return bool(self.table)

    def expected_per_tile(self, positions: int) -> float:
        """Terms a tile of `positions` bytes is expected to run, taking the text to be uniform
        over the estimated alphabet (the bytes of the program's narrow classes)."""
        if _n(self.alphabet) == 0:
            return 0.0
        e = 0.0
        for r, w in enumerate(self.windows[:self.n_terms]):
            if w is None:
                e += 1.0
            else:
                e += min(1.0, w.exact_chance(self.alphabet) * positions / self.stride)
        return e

    def mask_key(self, key: int) -> int:
        return key & ((1 << (8 * self.q)) - 1)

    def lookup_keys(self, key: int) -> List[int]:
        """The table keys a probe of q-gram `key` looks up: itself, and with its oldest /
        newest byte zeroed when the table holds wildcard grams of that kind."""
        key = self.mask_key(key)
        ks = [key]
        if self.wild_old:
            ks.append(key & ~0xFF)
        if self.wild_new:
            ks.append(key & ((1 << (8 * (self.q - 1))) - 1))
        return ks

    def match(self, key: int, pre3: int) -> int:
        """Bits set by q-gram `key` when the three bytes before it, packed like the records
        (the nearest in bits 0-7), are `pre3`."""
        m = 0
        for k in self.lookup_keys(key):
            m |= self.table.get(k, 0)
            for b, n, bit in self.ext.get(k, ()):
                mask = (1 << (8 * n)) - 1
                if (pre3 ^ b) & mask == 0:
                    m |= 1 << bit
        return m

    def bloom_keys(self) -> int:
        return len(self.table) + 255 * (len(self.wild_old) + len(self.wild_new))

    def always_mask(self) -> int:
        m = 0
        for r, z in enumerate(self.term_node):
            if z is None:
                m |= 1 << r
        for k, z in enumerate(self.pre_node):
            if z is None:
                m |= 1 << (self.n_terms + k)
        return m

    def bloom(self, bits: int = BLOOM_BITS) -> List[int]:
        assert 10 <= bits <= 24
        words = [0] * ((1 << bits) // 32)
        top = 8 * (self.q - 1)
        for key in self.table:
            variants = [key]
            if key in self.wild_old:
                variants += [(key & ~0xFF) | b for b in range(256)]
            if key in self.wild_new:
                variants += [(key & ~(0xFF << top)) | (b << top) for b in range(256)]
            for k in variants:
                h = bloom_hash(k, bits, self.q)
                words[h >> 5] |= 1 << (h & 31)
        return words

    def records(self, key: int) -> List[Tuple[int, int, int]]:
        """The records of q-gram `key`: (bytes, count, bit), the bit set when the first
        `count` bytes before the q-gram equal `bytes` (count 0: always)."""
        m = self.table.get(key, 0)
        base = [(0, 0, b) for b in range(self.n_bits) if (m >> b) & 1]
        return base + list(self.ext.get(key, []))

    def exact(self) -> Tuple[int, List[int], List[int], List[int]]:
        """(log2 slots, keys, slot info, records): open addressing with linear probing; a slot
        holds the key and its info word record_start << 8 | record_count (0 = empty slot, a
        key has at least one record); a record is two words, bytes | count << 24 and the bit it
        sets (see `records`).  All of it fits the kernel's shared memory."""
        n = len(self.table)
        log2 = 4
        while (1 << log2) < (3 * max(1, n) + 1) // 2:     # at most two thirds full
            log2 += 1
        slots = 1 << log2
        keys = [0] * slots
        info = [0] * slots
        recs: List[int] = []
        for key in sorted(self.table):
            s = exact_hash(key, log2)
            while info[s]:
                s = (s + 1) & (slots - 1)
            keys[s] = key
            rs = self.records(key)
            assert 0 < len(rs) < 256 and len(recs) // 2 < (1 << 23)
            info[s] = ((len(recs) // 2) << 8) | len(rs)
            for b, cnt, bit in rs:
                recs += [b | (cnt << 24), bit]
        return log2, keys, info, recs or [0, 0]


def _choose(gen, terms, pre, q, stride, PB, bloom_bits):
    """Filters of one configuration: (term windows/nodes, pre nodes, conditions, alphabet)."""
    d = gen.d
    wins = windows(gen, PB, q, stride)
    Z = zero_sets(gen, wins)
    # through a pre-pass addition a filter holds only while that addition's carry-in is zero,
    # which a '.*' after its first match almost never is; other additions are checked anyway
    Zp = zero_sets(gen, wins, blocked=frozenset(pre))
    # the text's alphabet, as the program sees it: the bytes its windows' narrow sets name
    # (a wide set such as '.' says nothing about the text)
    alpha = 0
    for ws in wins.values():
        for w in ws:
            for g in w.grams:
                for x in g:
                    if _n(x) <= 64:
                        alpha |= x
    bloom_p = 1.0 / (1 << bloom_bits)

    def score(w: Window) -> float:
        # chance hits of the exact records plus the Bloom false hits the keys add (per probe)
        return w.exact_chance(alpha) + (w.chance(alpha) + w.keys() * bloom_p) * COST_HIT / COST_RUN

    def best(zs):
        cands = [(score(w), z, w) for z in zs for w in wins[z]]
        if not cands:
            return None, None
        sc, z, w = min(cands, key=lambda c: (c[0], c[1]))
        return z, w

    term_node, term_win, term_cond = [], [], []
    for v in terms:
        z, w = best(Zp.get(v, ()))
        cond = z is None
        if z is None:
            z, w = best(Z.get(v, ()))
        term_node.append(z)
        term_win.append(w)
        term_cond.append(cond and z is not None)
    pre_node, pre_win = [], []
    for a in pre:
        z, w = best(Z.get(d.nodes[a].args[0], ()))
        pre_node.append(z)
        pre_win.append(w)
    return term_node, term_win, term_cond, pre_node, pre_win, alpha


def build(gen, terms: Sequence[int], pre: Sequence[int], key_limit: int = 1 << 16,
          config: Optional[Tuple[int, int]] = None, bloom_bits: int = BLOOM_BITS) -> TermFilter:
    """Filters for `terms` (node ids, in bit order) and pre-pass additions `pre` (node ids, in
    index order), in the configuration (q, stride) of lowest estimated cost per tile (or the
    one given)."""
    PB = position_bounds(gen)
    best_f, best_cost = None, None
    positions = 1024
    for q, stride in ([config] if config else CONFIGS):
        tn, tw, tc, pn, pw, alpha = _choose(gen, terms, pre, q, stride, PB, bloom_bits)
        f = TermFilter(len(terms), len(pre), tn, pn, tc, q=q, stride=stride, alphabet=alpha,
                       windows=tw + pw)
        table: Dict[int, int] = {}
        ext: Dict[int, List[Tuple[int, int, int]]] = {}
        wild = {WILD_OLD: set(), WILD_NEW: set()}
        for bit, w in enumerate(tw + pw):
            if w is None:
                continue
            for g, e in zip(w.grams, w.ext):
                packed = sum(b << (8 * i) for i, b in enumerate(e))
                kind = wildcard(g)
                for key in table_keys(g):
                    if kind:
                        wild[kind].add(key)
                    if e:
                        table.setdefault(key, 0)
                        ext.setdefault(key, []).append((packed, len(e), bit))
                    else:
                        table[key] = table.get(key, 0) | (1 << bit)
        if len(table) > key_limit or any(
                bin(table.get(k, 0)).count("1") + len(ext.get(k, [])) > 255 for k in table):
            table, ext = {}, {}
        if not table:
            wild = {WILD_OLD: set(), WILD_NEW: set()}
        f.table, f.ext = table, ext
        f.wild_old, f.wild_new = frozenset(wild[WILD_OLD]), frozenset(wild[WILD_NEW])
        if not f.enabled:
            continue
        # per tile of `positions` bytes (a warp of 32 lanes): probes per lane, slow-path hits
        # (Bloom false hits and chance q-grams), terms run
        hits = positions / stride * (f.bloom_keys() / (1 << bloom_bits)
                                     + sum(w.chance(alpha) for w in tw + pw if w is not None))
        cost = (positions / 32 / stride * COST_PROBE + hits * COST_HIT
                + f.expected_per_tile(positions) * COST_RUN)
        f.cost, f.hits = cost, hits
        if best_cost is None or cost < best_cost:
            best_f, best_cost = f, cost
    if best_f is None:
        q, stride = config or CONFIGS[-1]
        tn = [None] * len(terms)
        best_f = TermFilter(len(terms), len(pre), tn, [None] * len(pre), [False] * len(terms),
                            q=q, stride=stride, windows=[None] * (len(terms) + len(pre)))
    return best_f
