"""Trigram prefilter: which terms of a program can be non-zero in a tile, decided from the
tile's bytes before any bitstream is computed.

A *trigram node* is a node z whose set bits constrain the bytes at and just before them: if z
is set at position p, then bytes p-2, p-1 and p lie in sets S0, S1 and S2 (position bounds,
derived through AND, OR and Advance; see ``position_bounds``).  So when no trigram of
S0 x S1 x S2 occurs among the bytes a warp computes, z is zero in all of the warp's exact
lanes.  A node that bounds only its last two bytes is a bigram node: S0 is then every byte.

Zero implication.  Z(v) is the set of trigram nodes whose being zero makes v zero: AND and
Advance / Lookahead inherit the union of their operands' sets, OR / XOR / SEL the intersection,
and an addition its marker's set.  The last rule holds only while no carry enters the tile, so
the kernel also runs a term whenever one of its additions could take or owe a carry: a
look-back addition whose class is all ones at its carry lane or at its successor's, or a
pre-pass addition with a carry-in when the term's filter holds only through it.

Each term (an OR-ed leaf of an output) gets the most selective trigram node of Z(term) as its
filter, preferring one that does not pass through a pre-pass addition; a term without one
always runs.  Each pre-pass addition gets the filter of its marker,
so the pre-pass can skip the marker's computation too.

Extensions.  Where the filter node's bounds also fix single bytes 3, 4 and 5 positions back,
the trigram alone would pass the term on every chance occurrence of its last three bytes; the
table then holds, under the trigram, an extension record (those bytes and the term's bit), and
the kernel sets the bit only when the bytes before the trigram match.  On printable text this
makes the chance hits of literal filters about a hundred times rarer per byte of extension.

The kernel tests every trigram of the tile against a Bloom bitmap (2^20 bits by default, in
shared memory: a warp takes the slow path whenever any of its 32 lanes hits, so the bitmap is
sized for a per-lane false-hit rate well below 1/32) and resolves the rare hits in an exact open-addressed table that maps a trigram to the bit mask
of the filters containing it.  Both tables are generated here and compiled into the kernel.
"""

from __future__ import annotations

from dataclasses import dataclass, field
from typing import Dict, FrozenSet, List, Optional, Sequence, Tuple

ALL = (1 << 256) - 1
MAX_SET = 4096          # largest trigram set one filter may carry
MAX_EXT = 3             # bytes before the trigram an extension record may fix
EXT_DEPTH = 3 + MAX_EXT
BLOOM_BITS = 20         # log2 of the Bloom bitmap size (128 KB of shared memory)
HASH_BLOOM = 0x9E3779B1
HASH_EXACT = 0x85EBCA6B


def bloom_hash(key: int, bits: int = BLOOM_BITS) -> int:
    """Bit index of trigram `key` in a 2^bits-bit Bloom bitmap: the top `bits` bits of the 24-bit
    product key * HASH_BLOOM mod 2^24 (the kernel's bg_device.cuh bloom_probe)."""
    return ((key * HASH_BLOOM) & 0xFFFFFF) >> (24 - bits)


def exact_hash(key: int, log2_slots: int) -> int:
    return ((key * HASH_EXACT) & 0xFFFFFFFF) >> (32 - log2_slots)


def _bytes(s: int) -> List[int]:
    return [b for b in range(256) if (s >> b) & 1]


def position_bounds(gen, depth: int = 3) -> Dict[int, Tuple[int, ...]]:
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


def trigram_nodes(gen, PB: Dict[int, Tuple[int, ...]]) -> Dict[int, Tuple[int, int, int]]:
    """Trigram nodes of the live program and their byte sets (S0, S1, S2): every heavy node
    whose bounds at the last three positions are all constrained, with a small product."""
    d = gen.d
    out: Dict[int, Tuple[int, int, int]] = {}
    for z in sorted(gen.live):
        if d.is_cc(z):
            continue
        s2, s1, s0 = PB[z][0], PB[z][1], PB[z][2]
        if ALL in (s1, s2):
            continue
        # a bigram node (only its last two bytes bounded) is the trigram set ALL x S1 x S2
        size = bin(s0).count("1") * bin(s1).count("1") * bin(s2).count("1")
        if 0 < size <= MAX_SET:
            out[z] = (s0, s1, s2)
    return out


def zero_sets(gen, tri: Dict[int, Tuple[int, int, int]],
              blocked=frozenset()) -> Dict[int, FrozenSet[int]]:
    """Z(v) for every live node.  The result of an addition in `blocked` implies nothing (its
    carry may be non-zero whatever its marker)."""
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


def _set_size(sets: Tuple[int, int, int]) -> int:
    n = 1
    for x in sets:
        n *= bin(x).count("1")
    return n


def trigram_set(sets: Tuple[int, int, int]) -> List[int]:
    s0, s1, s2 = (_bytes(s) for s in sets)
    return [a | (b << 8) | (c << 16) for a in s0 for b in s1 for c in s2]


@dataclass
class TermFilter:
    """Per-program prefilter: bit r (r < n_terms) = term r may be non-zero, bit n_terms + k =
    pre-pass addition k's marker may be non-zero.  ``always`` holds the terms without a filter."""
    n_terms: int
    n_pre: int
    term_node: List[Optional[int]]
    pre_node: List[Optional[int]]
    term_cond: List[bool] = field(default_factory=list)  # filter implies zero only if no carry
    table: Dict[int, int] = field(default_factory=dict)   # trigram -> bits it sets by itself
    # trigram -> extension records (bytes 3, 4, 5 positions back packed low byte first, their
    # number, bit): the bit is set when those bytes precede the trigram
    ext: Dict[int, List[Tuple[int, int, int]]] = field(default_factory=dict)

    @property
    def n_bits(self) -> int:
        return self.n_terms + self.n_pre

    @property
    def words(self) -> int:
        return max(1, (self.n_bits + 31) // 32)

    @property
    def enabled(self) -> bool:
        return bool(self.table)

    alphabet: int = 0                                     # estimated text alphabet (bit set)
    sets: List[Optional[Tuple[int, int, int]]] = field(default_factory=list)

    def expected_per_tile(self, positions: int) -> float:
        """Terms a tile of `positions` bytes is expected to run, taking the text to be uniform
        over the estimated alphabet (the bytes of the program's narrow classes)."""
        a = self.alphabet
        na = bin(a).count("1")
        if na == 0:
            return 0.0
        e = 0.0
        for r, z in enumerate(self.term_node):
            if z is None or self.sets[r] is None:
                e += 1.0
                continue
            p = 1.0
            for s in self.sets[r]:
                p *= bin(s & a).count("1") / na
            e += min(1.0, p * positions)
        return e

    def match(self, trigram: int, pre3: int) -> int:
        """Bits set by `trigram` when the three bytes before it, packed like the records
        (byte 3 back in bits 0-7), are `pre3`."""
        m = self.table.get(trigram, 0)
        for b, n, bit in self.ext.get(trigram, ()):
            mask = (1 << (8 * n)) - 1
            if (pre3 ^ b) & mask == 0:
                m |= 1 << bit
        return m

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
        assert 5 < bits <= 24, "the Bloom index comes from a 24-bit product"
        words = [0] * ((1 << bits) // 32)
        for key in self.table:
            h = bloom_hash(key, bits)
            words[h >> 5] |= 1 << (h & 31)
        return words

    def records(self, key: int) -> List[Tuple[int, int, int]]:
        """The records of trigram `key`: (bytes, count, bit), the bit set when the first
        `count` bytes before the trigram equal `bytes` (count 0: always)."""
        m = self.table.get(key, 0)
        base = [(0, 0, b) for b in range(self.n_bits) if (m >> b) & 1]
        return base + list(self.ext.get(key, []))

    def exact(self) -> Tuple[int, List[int], List[int], List[int]]:
        """(log2 slots, keys, slot info, records): open addressing with linear probing; a key
        slot holds trigram | 1 << 31 (0 = empty) and its info word record_start << 8 |
        record_count; a record is two words, bytes | count << 24 and the bit it sets (see
        `records`).  All of it fits the kernel's shared memory."""
        n = len(self.table)
        log2 = 4
        while (1 << log2) < 2 * max(1, n):
            log2 += 1
        slots = 1 << log2
        keys = [0] * slots
        info = [0] * slots
        recs: List[int] = []
        for key in sorted(self.table):
            s = exact_hash(key, log2)
            while keys[s]:
                s = (s + 1) & (slots - 1)
            keys[s] = key | (1 << 31)
            rs = self.records(key)
            assert len(rs) < 256 and len(recs) // 2 < (1 << 23)
            info[s] = ((len(recs) // 2) << 8) | len(rs)
            for b, cnt, bit in rs:
                recs += [b | (cnt << 24), bit]
        return log2, keys, info, recs or [0, 0]

def build(gen, terms: Sequence[int], pre: Sequence[int], tri_limit: int = 1 << 16) -> TermFilter:
    """Filters for `terms` (node ids, in bit order) and pre-pass additions `pre` (node ids, in
    index order)."""
    tri = trigram_nodes(gen, position_bounds(gen))
    Z = zero_sets(gen, tri)
    # through a pre-pass addition a filter holds only while that addition's carry-in is zero,
    # which a '.*' after its first match almost never is; other additions are checked anyway
    Zp = zero_sets(gen, tri, blocked=frozenset(pre))
    d = gen.d
    deep = position_bounds(gen, depth=EXT_DEPTH)

    def fixed_before(z) -> List[int]:
        """Single bytes that the bounds of z fix 3, 4, 5 positions back (stopping at the
        first position that is not a single byte)."""
        out = []
        for k in range(3, EXT_DEPTH):
            s = deep[z][k]
            if s == ALL or bin(s).count("1") != 1:
                break
            out.append(s.bit_length() - 1)
        return out

    def best(zs) -> Optional[int]:
        # smallest trigram set, then the longest extension (fewest chance hits)
        cands = sorted(zs, key=lambda z: (_set_size(tri[z]), -len(fixed_before(z)), z))
        return cands[0] if cands else None

    term_node, term_cond = [], []
    for v in terms:
        z = best(Zp.get(v, ()))
        cond = z is None
        if z is None:
            z = best(Z.get(v, ()))
        term_node.append(z)
        term_cond.append(cond and z is not None)
    pre_node = [best(Z.get(d.nodes[a].args[0], ())) for a in pre]
    f = TermFilter(len(terms), len(pre), term_node, pre_node, term_cond)
    f.sets = [tri[z] if z is not None else None for z in term_node]
    # the text's alphabet, as the program sees it: the bytes its filters name
    alpha = 0
    for s in f.sets:
        for x in s or ():
            if x != ALL:
                alpha |= x
    f.alphabet = alpha
    table: Dict[int, int] = {}
    ext: Dict[int, List[Tuple[int, int, int]]] = {}
    for bit, z in list(enumerate(term_node)) + [(len(terms) + k, z) for k, z in enumerate(pre_node)]:
        if z is None:
            continue
        fixed = fixed_before(z)
        packed = sum(b << (8 * i) for i, b in enumerate(fixed))
        for key in trigram_set(tri[z]):
            if fixed:
                table.setdefault(key, 0)
                ext.setdefault(key, []).append((packed, len(fixed), bit))
            else:
                table[key] = table.get(key, 0) | (1 << bit)
    if len(table) > tri_limit or any(
            bin(table.get(k, 0)).count("1") + len(ext.get(k, [])) > 255 for k in table):
        table, ext = {}, {}
    f.table = table
    f.ext = ext
    return f
