"""CPU checks of the q-gram prefilter (bitgen_gb300/prefilter.py).

Soundness: a term that is non-zero in a tile's exact lanes must have its bit set by the tile's
q-gram scan.  The scan is simulated here exactly as the kernel does it (every q-gram lying
wholly inside the bytes the warp computes and ending at a probed position, looked up in the
exact table), and the per-regex streams come from the C oracle.  Terms behind an addition are
excluded, since the kernel runs those on its own carry checks.  The Bloom bitmap must contain
every key of the exact table (the table only removes Bloom false positives), and the table's
probes must find every key.  Every configuration (q-gram length, stride) is checked.
"""

import numpy as np
import pytest

from bitgen_gb300 import prefilter, workloads
from bitgen_gb300.compiler import ADD_OPS, Tuning, _Gen, build_dag
from bitgen_gb300.regex import compile_group
from oracle import cpu


def _setup(patterns, n_groups, per_regex=True, wpt=2, config=None):
    groups = [compile_group(g) for g in patterns.groups(n_groups)]
    dag, outs, names = build_dag(groups, per_regex)
    gen = _Gen(dag, Tuning(wpt=wpt))
    gen.analyse(outs)
    terms = [(leaf, o) for o, v in enumerate(outs) for leaf in gen.or_leaves(v)]
    pre = [v for v, _ in sorted(gen.pre.items(), key=lambda x: x[1])]
    f = prefilter.build(gen, [v for v, _ in terms], pre, config=config)
    return groups, gen, terms, f


def _lookup1(key, pre3, log2, keys, info, recs):
    """The kernel's exact lookup of one key (bg_device.cuh qgram_exact), over the generated
    tables."""
    s = prefilter.exact_hash(key, log2)
    for _ in range(len(keys)):
        if info[s] == 0:
            return 0
        if keys[s] == key:
            m = 0
            e = info[s]
            for i in range(e >> 8, (e >> 8) + (e & 255)):
                r, bit = recs[2 * i], recs[2 * i + 1]
                cmp = (1 << (8 * (r >> 24))) - 1
                if (pre3 ^ r) & cmp == 0:
                    m |= 1 << bit
            return m
        s = (s + 1) & (len(keys) - 1)
    return 0


def _lookup(f, key, pre3, *tabs):
    """A Bloom hit's lookups (resolve_hits): the q-gram itself, and with its oldest / newest
    byte zeroed when the table holds wildcard q-grams of that kind."""
    key = f.mask_key(key)
    m = _lookup1(key, pre3, *tabs)
    if f.wild_old:
        m |= _lookup1(key & ~0xFF, pre3, *tabs)
    if f.wild_new:
        m |= _lookup1(key & ((1 << (8 * (f.q - 1))) - 1), pre3, *tabs)
    return m


def _found(f, key):
    return any(k in f.table for k in f.lookup_keys(key))


@pytest.mark.parametrize("config", prefilter.CONFIGS)
def test_tables_are_consistent(config):
    _, _, _, f = _setup(workloads.throughput_patterns(seed=3, n=64), 4, config=config)
    assert f.enabled and f.ext and (f.q, f.stride) == config
    bloom = f.bloom()
    tabs = f.exact()
    rng = np.random.default_rng(5)
    for key, m in f.table.items():
        h = prefilter.bloom_hash(key, q=f.q)
        assert (bloom[h >> 5] >> (h & 31)) & 1
        if f.q == 3:   # the byte above a trigram does not move its Bloom bit
            assert prefilter.bloom_hash(key | 0xAB000000, q=3) == h
        recs = f.ext.get(key, [])
        pres = [int(x) for x in rng.integers(0, 1 << 24, size=4)] + [b for b, _, _ in recs]
        for pre3 in pres:
            assert _lookup(f, key, pre3, *tabs) == f.match(key, pre3)
        assert _lookup(f, key, 0, *tabs) & m == m
    absent = 0x7f7f7f7f & ((1 << (8 * f.q)) - 1)
    assert _lookup(f, absent, 0, *tabs) == 0 or absent in f.table


def _probe_hits(f, text):
    """Per position p: the bits the kernel's probe of the q-gram ending at p sets (0 where p is
    not probed), given that the warp's bytes start at or before p - q - 2."""
    n = text.size
    b = text.astype(np.int64)
    key = np.zeros(n, dtype=np.int64)
    for i in range(f.q):
        key[f.q - 1:] |= b[i:n - f.q + 1 + i] << (8 * i)
    pre3 = np.zeros(n, dtype=np.int64)          # the three bytes before it, nearest first
    for d in range(3):
        pre3[f.q + d:] |= b[:n - f.q - d] << (8 * d)
    probed = (np.arange(n) % f.stride) == f.stride - 1
    probed[:f.q - 1] = False
    hit = np.zeros(n, dtype=object)
    ks = np.array(sorted(f.table), dtype=np.int64)
    cand = np.isin(key, ks)
    if f.wild_old:
        cand |= np.isin(key & ~0xFF, ks)
    if f.wild_new:
        cand |= np.isin(key & ((1 << (8 * (f.q - 1))) - 1), ks)
    cand &= probed
    for p in np.nonzero(cand)[0]:
        hit[p] = f.match(int(key[p]), int(pre3[p]))
    return key, pre3, probed, hit


class _EmitterPatterns:
    """Lookarounds, loop-free group stars, wide repeats and end assertions inside patterns."""
    regexes = [r"abcd(?=x)", r"qrst(?!u)", r"(?<=ab)cdqx", r"xyzq(ab|cde)*f", r"mnop(rs)+t",
               r"hijk.{0,40}lmno", r"wxyz[0-9]{16}", r"klmn$\nopq", r"(?<![0-9])1234(?![0-9])",
               r"efgh(ij){2,20}kl"]
    witnesses = [b"abcdx", b"qrstv", b"abcdqx", b"xyzqabcdecdef", b"mnoprsrsrst",
                 b"hijk" + b"." * 30 + b"lmno", b"wxyz" + b"5" * 16, b"klmn\nopq", b" 1234 ",
                 b"efgh" + b"ij" * 5 + b"kl"]

    def groups(self, n):
        return [self.regexes[i::n] for i in range(n)]


class _FlagPatterns:
    """Word boundaries and case-insensitive groups (PCRE-style rule fragments), with witnesses."""
    regexes = [r"\bhello\w+world\b", r"(?i)\bselect\s+\*\s+from\b", r"\Bing\b",
               r"\bzq\d{2,5}\b", r"(?i)passwd", r"x(?i:ab)y\B", r"\b[a-c]{3}\b",
               r"(?i)\bget /[a-z]+\.php"]
    witnesses = [b" helloXworld ", b" SeLeCt * FROM ", b"ringing ", b" zq123 ", b"PassWD",
                 b"xABya", b" abc ", b" gEt /index.php"]

    def groups(self, n):
        return [self.regexes[i::n] for i in range(n)]


@pytest.mark.parametrize("wpt,kind,config", [(1, "throughput", None), (2, "throughput", (4, 2)),
                                             (1, "throughput", (4, 1)), (2, "throughput", (3, 1)),
                                             (2, "dna", None), (1, "flags", None),
                                             (1, "emitter", None), (2, "emitter", (4, 2))])
def test_prefilter_is_sound(wpt, kind, config):
    """Also on IUPAC motifs over DNA text (the filter the split form would use there if forced;
    the compiler picks the single-kernel form for it), on word boundaries and case-insensitive
    groups, and on lookarounds, loop-free group stars and wide repeats."""
    n = 300_000
    if kind == "dna":
        ps = workloads.dna_motifs(24, seed=5)
        text = workloads.plant(workloads.dna_text(n, seed=43), ps.witnesses, 700, 42)
    elif kind == "flags":
        ps = _FlagPatterns()
        text = workloads.plant(workloads.printable_text(n, 44), ps.witnesses, 300, 45)
    elif kind == "emitter":
        ps = _EmitterPatterns()
        text = workloads.plant(workloads.printable_text(n, 46), ps.witnesses, 300, 47)
    else:
        ps = workloads.throughput_patterns(seed=3, n=64)
        text = workloads.plant(workloads.printable_text(n, 41), ps.witnesses, 700, 42)
    groups, gen, terms, f = _setup(ps, 4, wpt=wpt, config=config)
    if config:
        assert (f.q, f.stride) == config
    streams, _ = cpu.run_groups(groups, text, per_regex=True)
    hl, tl = gen.hl, gen.tl
    tile_words = (32 - hl - tl) * wpt
    W = (n + 31) // 32
    key, pre3, probed, hit_bits = _probe_hits(f, text)
    q = f.q
    has_add = [any(gen.d.nodes[a].op in ADD_OPS for a in gen.heavy_ancestors(v)) for v, _ in terms]
    by_out = {}
    for r, (v, o) in enumerate(terms):
        by_out.setdefault(o, []).append(r)
    checked = 0
    n_tiles = max(1, -(-W // tile_words))
    for g in range(n_tiles):
        base = g * tile_words - hl * wpt               # word index of lane 0, word 0
        lo_b = max(0, base * 32)
        hi_b = min(n, (base + 32 * wpt) * 32)
        cand = 0
        for p in range(lo_b + q - 1, hi_b):
            if not probed[p]:
                continue
            if p < lo_b + q + 2 and _found(f, int(key[p])):
                # bytes before the warp's first byte read as zero in the kernel
                keep = (1 << (8 * max(0, p - q + 1 - lo_b))) - 1
                cand |= f.match(int(key[p]), int(pre3[p]) & keep)
            elif hit_bits[p]:
                cand |= hit_bits[p]
        cand |= f.always_mask()
        ex_lo, ex_hi = max(0, g * tile_words), min(W, (g + 1) * tile_words)
        for o, rs in by_out.items():
            if any(has_add[r] for r in rs):
                continue
            if np.any(streams[o][ex_lo:ex_hi]):
                assert any((cand >> r) & 1 for r in rs), (g, o)
                checked += 1
    assert checked > 10
    # selective: on this text most tiles flag few terms
    assert sum(1 for r, z in enumerate(f.term_node) if z is None) < len(terms) // 4


def test_cost_model_prefers_four_byte_grams_on_the_benchmark_grammar():
    """The 256-regex workload's literals are 4-12 bytes: 4-grams, which are far rarer by chance
    than trigrams, cover every term."""
    _, _, terms, f = _setup(workloads.throughput_patterns(seed=3, n=256), 16, per_regex=False,
                            wpt=1)
    assert f.q == 4 and f.always_mask() == 0
    tri = _setup(workloads.throughput_patterns(seed=3, n=256), 16, per_regex=False, wpt=1,
                 config=(3, 1))[3]
    assert f.cost < tri.cost


def test_form_follows_expected_selectivity():
    """On printable text the 256-regex program's filters pass few terms per tile (split form);
    on a 4-letter DNA text nearly every motif's trigrams occur in every tile (single form)."""
    from bitgen_gb300.compiler import generate_kernel
    thr = [compile_group(g) for g in workloads.throughput_patterns(seed=3, n=256).groups(16)]
    dna = [compile_group(g) for g in workloads.dna_motifs(64, seed=5).groups(4)]
    assert generate_kernel(thr, Tuning()).n_parts > 0
    assert generate_kernel(dna, Tuning()).n_parts == 0
    # the limit can force either form
    assert generate_kernel(dna, Tuning(prefilter_limit=2.0)).n_parts > 0
    assert generate_kernel(thr, Tuning(prefilter_limit=0.0)).n_parts == 0


def test_large_programs_fit_classify_shared_memory():
    """1024 regexes: the classify block shrinks (and then the Bloom bitmap) until its shared
    memory fits one block."""
    import re
    from bitgen_gb300.compiler import generate_kernel
    gs = [compile_group(g) for g in workloads.throughput_patterns(seed=83, n=1024).groups(16)]
    spec = generate_kernel(gs, Tuning())
    block, smem = map(int, re.search(r"bg_cls_cfg\[2\] = \{(\d+)u, (\d+)u\}", spec.source).groups())
    assert smem <= 227 * 1024 and block % 32 == 0 and spec.n_parts > 0


def test_parts_inline_up_to_the_threshold():
    """Up to Tuning.inline_parts parts are inlined into the execute kernel (one whole-program
    compile: no part sections, a switch); more parts are separate sections called through a
    table."""
    from bitgen_gb300.compiler import generate_kernel
    gs = [compile_group(g) for g in workloads.throughput_patterns(seed=3, n=64).groups(4)]
    inl = generate_kernel(gs, Tuning())
    assert 0 < inl.n_parts <= Tuning().inline_parts
    assert inl.source.count("//@@BG_PART") == 1 and "bg_part_tab" not in inl.source
    assert "static __device__ __forceinline__ void bg_part_0(" in inl.source
    sep = generate_kernel(gs, Tuning(inline_parts=0))
    assert sep.source.count("//@@BG_PART") == sep.n_parts + 1 and "bg_part_tab[k](" in sep.source


def test_split_form_part_outputs():
    """The split form records which outputs each part writes (read with the work counters):
    every output is written by some part, every part writes at least one output, and with
    merged outputs each part holds at most part_cap terms, so at most that many outputs."""
    from bitgen_gb300.compiler import generate_kernel
    gs = [compile_group(g) for g in workloads.throughput_patterns(seed=3, n=256).groups(16)]
    spec = generate_kernel(gs, Tuning())
    assert spec.n_parts == len(spec.part_outputs) > 0
    assert sorted({o for outs in spec.part_outputs for o in outs}) == list(range(spec.n_outputs))
    assert all(0 < len(outs) <= 2 for outs in spec.part_outputs)
    assert generate_kernel(gs, Tuning(prefilter_limit=0.0)).part_outputs == []


def test_wildcard_grams_cover_four_byte_literals_at_stride_two():
    """At stride 2 a four-byte literal has, in one phase, only three known bytes in the probed
    4-gram: such grams are registered with a free oldest or newest byte, so that no term of the
    256-regex workload is left without a filter; the Bloom bitmap holds all 256 variants of
    each, and the lookups of every variant find the gram's records."""
    _, _, terms, f = _setup(workloads.throughput_patterns(seed=3, n=256), 16, per_regex=False,
                            wpt=1, config=(4, 2))
    assert f.always_mask() == 0 and (f.wild_old or f.wild_new)
    bloom = f.bloom()
    tabs = f.exact()
    top = 8 * (f.q - 1)
    for key in sorted(f.wild_old | f.wild_new)[:6]:
        want = f.table[key]
        for b in (0, 1, 0x41, 0xFF):
            for v, ok in (((key & ~0xFF) | b, key in f.wild_old),
                          ((key & ~(0xFF << top)) | (b << top), key in f.wild_new)):
                if not ok:
                    continue
                h = prefilter.bloom_hash(v, q=f.q)
                assert (bloom[h >> 5] >> (h & 31)) & 1
                assert _lookup(f, v, 0, *tabs) & want == want == f.match(v, 0) & want
    assert prefilter.wildcard((prefilter.ALL, 1, 2, 4)) == prefilter.WILD_OLD
    assert prefilter.wildcard((1, 2, 4, prefilter.ALL)) == prefilter.WILD_NEW
    assert prefilter.wildcard((1, prefilter.ALL, 2, 4)) < 0
    assert prefilter.wildcard((prefilter.ALL, 2, 4)) < 0    # trigrams keep every byte
