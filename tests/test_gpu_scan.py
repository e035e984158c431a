"""GPU parity: the fused sm_103a scan kernels and the whole-stream executor against the oracle.

Every comparison is bit-exact (integer work): output streams in the reference layout and their
popcounts.  Inputs are seeded; sizes keep the big-integer oracle within seconds.
"""

import json
import os

import numpy as np
import pytest
import torch

from bitgen_gb300.compiler import Tuning
from bitgen_gb300.engine import Program, basis_input, pack_bytes, transpose
from bitgen_gb300.pablo import parse_pablo
from bitgen_gb300.refir import group_from_ir
from bitgen_gb300.regex import compile_group
from bitgen_gb300 import workloads
from oracle.pablo_ref import transpose_ref
from tests.helpers import first_diff, oracle_streams, rand_text

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def check(prog: Program, groups, items, per_regex=False):
    inp = pack_bytes(items)
    res = prog.scan(inp)
    torch.cuda.synchronize()
    streams = res.streams.cpu().numpy()
    counts = res.counts.cpu().numpy()
    for i, data in enumerate(items):
        data = np.asarray(data, dtype=np.uint8)
        want = oracle_streams(groups, data, per_regex)
        assert len(want) == prog.n_outputs
        o = res.word_offsets[i]
        W = res.words[i]
        for k, w in enumerate(want):
            got = streams[k, o:o + W]
            d = first_diff(got, w)
            assert d is None, f"input {i} (n={data.size}) output {k}: {d}"
            assert counts[k, i] == int(np.unpackbits(w.view(np.uint8)).sum())


SMALL = None


def small():
    global SMALL
    if SMALL is None:
        ps, text = workloads.small_workload()
        groups = [compile_group(g) for g in ps.groups(4)]
        SMALL = (ps, text, groups)
    return SMALL


@pytest.mark.parametrize("wpt,skip,block,extra", [(1, 1, 256, {}), (2, 1, 256, {}), (4, 1, 128, {}),
                                                  (2, 0, 64, {}), (2, 3, 256, {}),
                                                  (2, 1, 256, {"lockstep": True}),
                                                  (2, 1, 256, {"edge_variants": True, "part_cap": 4}),
                                                  (2, 1, 256, {"prefilter": False}),
                                                  (1, 1, 256, {"part_cap": 1}),
                                                  (1, 1, 256, {"merge_outputs": False}),
                                                  (1, 1, 256, {"part_cap": 2}),
                                                  (2, 1, 256, {"carry_prepass": False})])
def test_small_workload_tunings(cuda, wpt, skip, block, extra):
    ps, text, groups = small()
    prog = Program(groups, tuning=Tuning(wpt=wpt, skip_interval=skip, block=block, **extra))
    check(prog, groups, [text])
    prog.close()


def test_small_workload_per_regex(cuda):
    ps, text, groups = small()
    prog = Program(groups, per_regex=True)
    check(prog, groups, [text], per_regex=True)


def test_ragged_lengths_and_tile_edges(cuda):
    groups = [compile_group(["ab[0-9]*c", "x.{2,4}y"]), compile_group(["q+", "[^a-m]z"])]
    prog = Program(groups, tuning=Tuning(wpt=1))
    tile_chars = prog.spec.tile_words * 32
    lens = list(range(0, 70)) + [tile_chars + d for d in (-33, -32, -1, 0, 1, 31, 32, 33)] + \
        [3 * tile_chars + 7, 17 * tile_chars - 5]
    items = [rand_text(n, 100 + n, b"abcqxyz0123\n") for n in lens]
    check(prog, groups, items)


def test_long_carries_across_many_tiles(cuda):
    # '.*' on text without LF: one early prefix match turns every later position on
    groups = [compile_group(["k9.*zz"]), compile_group(["a[ab]*b", "c[^d]*e"])]
    n = 300_000
    t = rand_text(n, 7, b"abcefgh")
    t[5:7] = np.frombuffer(b"k9", np.uint8)
    t[-3:] = np.frombuffer(b"zz ", np.uint8)
    t2 = np.full(n, ord("a"), np.uint8)  # one 'a' run spanning every tile, 'b' at the end
    t2[-1] = ord("b")
    for tun in (Tuning(wpt=1), Tuning(wpt=4, block=128), Tuning(lockstep=True),
                Tuning(edge_variants=True), Tuning(carry_prepass=False), Tuning(prefilter=False)):
        prog = Program(groups, tuning=tun)
        check(prog, groups, [t, t2, t2[:1000], t[:5]])


def test_carry_prepass_matches_lookback_and_oracle(cuda):
    """Wide-class additions whose operands need no other addition ('.*', '[^x]*') take their
    carries from the pre-pass and the carry scan; nested ones ('m.*n.*o', second '.*') still use
    the look-back.  Both forms must agree with the oracle over many inputs in one launch (the
    carry restarts at every input, including inputs that start inside one scan thread's run of
    tiles) and over a long input."""
    groups = [compile_group(["k9.*zz", "q[^x]*r"]), compile_group(["m.*n.*o"]), compile_group(["ab+c"])]
    rng = np.random.default_rng(5)
    items = [rand_text(int(n), 100 + i, b"kz9qrmnoabcx ") for i, n in
             enumerate(rng.integers(0, 3000, size=300))]
    long = rand_text(2_000_003, 9, b"abcdefghijklmnopqrstuvwyz ")
    long[10:12] = np.frombuffer(b"k9", np.uint8)
    long[1_999_990:1_999_992] = np.frombuffer(b"zz", np.uint8)
    items.append(long)
    with_pre = Program(groups)
    without = Program(groups, tuning=Tuning(carry_prepass=False, prefilter=False))
    assert with_pre.spec.n_pre >= 2 and without.spec.n_pre == 0
    assert with_pre.spec.n_pre < with_pre.spec.n_adds  # the nested '.*' is not pre-passed
    check(with_pre, groups, items)
    inp = pack_bytes(items)
    a, b = with_pre.scan(inp), without.scan(inp)
    torch.cuda.synchronize()
    assert torch.equal(a.counts, b.counts)
    for o, w in zip(a.word_offsets, a.words):  # padding words between inputs are not written
        assert torch.equal(a.streams[:, o:o + w], b.streams[:, o:o + w])


def test_scanthru_and_while_forms(cuda):
    src = """
lf = (basis4 & basis6)
a = (~basis0)
m = (a & basis1)
s = pablo.ScanThru(m, a)
st = pablo.MatchStar(m, lf)
r = (s | st)
output.matches = r
"""
    g = parse_pablo(src)
    items = [rand_text(n, n, bytes(range(0, 256))) for n in (1, 100, 5000, 70000)]
    check(Program([g]), [g], items)
    # icgrep's -disable-matchstar loop form compiles to MatchStar on the fused path and runs
    # literally on the whole-stream executor; both agree with the oracle
    gw = compile_group(["ab*c", "x[yz]*w", "[0-9]+k"], matchstar=False)
    items = [rand_text(n, n, b"abcxyzwk0123") for n in (10, 999, 40000)]
    fused = Program([gw])
    assert fused.fused
    check(fused, [gw], items)
    check(Program([gw], executor="interp"), [gw], items)
    # a loop over a multi-character group stays a loop: whole-stream executor
    gg = compile_group(["x(yz)*w", "a(bc)+d"], matchstar=False)
    prog = Program([gg])
    assert not prog.fused
    check(prog, [gg], [rand_text(n, n, b"abcdxyzw") for n in (1, 500, 20000)])


def test_reference_fixture_program_on_executor(cuda):
    with open(os.path.join(GOLDEN, "parser.json")) as f:
        ir = json.load(f)["reference_ir"]["xml_lexical_parsing"]
    g = group_from_ir(ir)
    prog = Program([g])
    assert not prog.fused  # its while loop is not a MatchStar loop: whole-stream semantics
    items = [np.frombuffer(b"<a<bcd<EFGH>x<yz>" * k, np.uint8) for k in (1, 7, 300)]
    items.append(rand_text(5000, 3, b"<>abAB xyz"))
    check(prog, [g], items)


def test_if_else_whole_stream(cuda):
    src = """
a = (basis1 & basis2)
b = (~basis3)
if a:
  x = pablo.Advance(a, 3)
else:
  x = b
y = (x | a)
output.matches = y
"""
    g = parse_pablo(src)
    items = [rand_text(100, 1, b"0123"), rand_text(100, 2, b"abcd"), rand_text(4000, 3)]
    check(Program([g]), [g], items)


def test_fused_equals_executor_on_throughput_patterns(cuda):
    ps = workloads.throughput_patterns(seed=3, n=48)
    groups = [compile_group(g) for g in ps.groups(4)]
    base = workloads.plant(workloads.printable_text(1 << 16, 4), ps.witnesses, 1024, 5)
    a = Program(groups)
    b = Program(groups, executor="interp")
    inp = pack_bytes([base])
    ra, rb = a.scan(inp), b.scan(inp)
    assert torch.equal(ra.streams, rb.streams)
    assert torch.equal(ra.counts, rb.counts)
    assert int(ra.counts.sum()) > 0


def test_basis_input_matches_bytes(cuda):
    ps, text, groups = small()
    prog = Program(groups)
    M = 3
    npad = -(-text.size // 32) * 32
    bytestream = torch.zeros((1, M, npad), dtype=torch.uint8, device=cuda)
    for m in range(M):
        bytestream[0, m, :text.size] = torch.from_numpy(np.roll(text, 97 * m).copy())
    basis = torch.zeros((1, M, 8, npad // 32), dtype=torch.uint32, device=cuda)
    transpose(bytestream, basis)
    res = prog.scan(basis_input(basis, [text.size] * M))
    for m in range(M):
        want = oracle_streams(groups, np.roll(text, 97 * m))
        for k, w in enumerate(want):
            assert first_diff(res.stream(k, m).cpu().numpy(), w) is None


def test_transpose_against_reference_vectors(cuda):
    gold = np.load(os.path.join(GOLDEN, "transpose.npz"))
    for k in gold.files:
        if not k.startswith("in"):
            continue
        src = gold[k]
        want = gold[k.replace("in", "out", 1)]
        arr = src if src.ndim == 2 else src[None]
        t = torch.from_numpy(arr.copy()).to(cuda)[None].contiguous()
        out = torch.zeros((1, arr.shape[0], 8, arr.shape[1] // 32), dtype=torch.uint32, device=cuda)
        transpose(t, out)
        assert np.array_equal(out.cpu().numpy().reshape(want.shape), want), k


@pytest.mark.parametrize("n,m", [(32, 1), (1 << 20, 1), (4096, 5), (96, 130)])
def test_transpose_random(cuda, n, m):
    rng = np.random.default_rng(n + m)
    a = rng.integers(0, 256, size=(m, n), dtype=np.uint8)
    t = torch.from_numpy(a).to(cuda)[None].contiguous()
    out = torch.zeros((1, m, 8, n // 32), dtype=torch.uint32, device=cuda)
    transpose(t, out)
    got = out.cpu().numpy()[0]
    for i in range(m):
        assert np.array_equal(got[i], transpose_ref(a[i])), i


def test_many_inputs_one_launch(cuda):
    ps = workloads.throughput_patterns(seed=11, n=24)
    groups = [compile_group(g) for g in ps.groups(3)]
    lens = workloads.batched_lengths(300, seed=12, median=900, lo=1, hi=5000)
    items = workloads.batched_inputs(lens, 13, ps.witnesses)
    check(Program(groups), groups, items)


def test_sparse_positions_match_streams(cuda):
    ps = workloads.throughput_patterns(seed=51, n=24)
    groups = [compile_group(g) for g in ps.groups(3)]
    lens = [0, 5, 4000, 70000, 33]
    items = [workloads.plant(workloads.printable_text(n, 52 + n), ps.witnesses, 512, 53 + n) for n in lens]
    prog = Program(groups)
    res = prog.scan(pack_bytes(items), positions=True)
    total = 0
    for i, data in enumerate(items):
        for o in range(prog.n_outputs):
            words = res.stream(o, i).cpu().numpy()
            bits = np.unpackbits(words.astype(">u4").view(np.uint8))
            want = np.nonzero(bits)[0]
            assert np.array_equal(res.match_positions(o, i), want), (i, o)
            total += want.size
    assert total == int(res.counts.sum()) > 0
    # a buffer that is too small is reported, counts stay exact
    from bitgen_gb300 import _native as N
    with pytest.raises(N.BitgenError) as e:
        prog.scan(pack_bytes(items), positions=True, pos_capacity=3)
    assert e.value.status == N.BG_ERR_CAPACITY


def test_counts_only_launches_of_merging_programs(cuda):
    """A program whose parts OR into shared outputs takes its counts from the bits each part
    adds, so a launch without output streams needs a position set: the C ABI rejects it with
    BG_ERR_INVALID until bg_plan_set_positions sized one, and the Python plan supplies its own
    streams.  Counts equal those of a launch with streams and those of the oracle."""
    import ctypes as C
    from bitgen_gb300 import _native as N
    ps, text, groups = small()
    prog = Program(groups)
    assert prog.merges
    inp = pack_bytes([text])
    a = prog.scan(inp, streams=False)
    b = prog.scan(inp)
    torch.cuda.synchronize()
    assert torch.equal(a.counts, b.counts)
    want = [int(np.unpackbits(w.view(np.uint8)).sum()) for w in oracle_streams(groups, text)]
    assert a.counts[:, 0].tolist() == want
    plan = prog.plan(inp, b.word_offsets, b.streams.shape[1])
    rc = N.lib().bg_plan_launch(plan._h, inp.data.data_ptr(), None, b.counts.data_ptr(), None)
    assert rc == N.BG_ERR_INVALID
    assert b"merges outputs across parts" in N.lib().bg_last_error()


def test_large_pattern_set_matches_c_oracle(cuda):
    """1024 regexes in 16 groups (the classify block and Bloom bitmap shrink to fit shared
    memory) over 1 MiB of printable text with planted matches, two ragged inputs."""
    from oracle import cpu
    ps = workloads.throughput_patterns(seed=83, n=1024)
    groups = [compile_group(g) for g in ps.groups(16)]
    prog = Program(groups)
    assert prog.fused and prog.spec.n_parts > 0
    a = workloads.plant(workloads.printable_text((1 << 20) + 77, 84), ps.witnesses, 2048, 85)
    b = a[: 50_001].copy()
    res = prog.scan(pack_bytes([a, b]))
    torch.cuda.synchronize()
    got = res.streams.cpu().numpy().view(np.uint32)
    for i, data in enumerate((a, b)):
        want, wc = cpu.run_groups(groups, data)
        o, W = res.word_offsets[i], res.words[i]
        for k, w in enumerate(want):
            d = first_diff(got[k, o:o + W], w)
            assert d is None, (i, k, d)
        assert res.counts[:, i].cpu().tolist() == wc
    assert int(res.counts.sum()) > 0


def test_work_counters(cuda):
    """`scan(stats=True)` reports, per part of a split-form program, the tiles the execute pass
    ran it on and the rows of its work list.  Every tile holding a match of an output ran a part
    that writes that output; a listed row has at least one such tile; the trigram filter keeps
    most parts off most tiles of printable text; a single-kernel program reports only its tiles."""
    ps = workloads.throughput_patterns(seed=91, n=64)
    groups = [compile_group(g) for g in ps.groups(4)]
    prog = Program(groups)
    assert prog.fused and prog.spec.n_parts > 0
    data = workloads.plant(workloads.printable_text((1 << 19) + 333, 92), ps.witnesses, 4096, 93)
    inp = pack_bytes([data])
    res = prog.scan(inp, stats=True)
    st = res.stats
    T = prog.tiles_for([data.size])
    R = -(-T // 32)
    assert st["form"] == "split" and st["tiles"] == T
    assert len(st["tiles_run"]) == len(st["rows"]) == len(st["part_outputs"]) == prog.spec.n_parts
    for k, (n, r) in enumerate(zip(st["tiles_run"], st["rows"])):
        assert 0 <= r <= R and r <= n <= min(T, 32 * r), (k, n, r)
    tw = prog.spec.tile_words
    streams = res.streams.cpu().numpy()
    for o in range(prog.n_outputs):
        bits = np.unpackbits(streams[o, :res.words[0]].astype(">u4").view(np.uint8))
        need = np.unique(np.nonzero(bits)[0] // 32 // tw).size
        ran = sum(n for n, outs in zip(st["tiles_run"], st["part_outputs"]) if o in outs)
        assert ran >= need, (o, ran, need)
    assert int(res.counts.sum()) > 0
    assert sum(st["tiles_run"]) <= 0.5 * T * prog.spec.n_parts
    # the counters read back do not disturb the next launch, which reports the same work
    again = prog.scan(inp, stats=True)
    assert again.stats == st
    assert all(torch.equal(again.stream(o), res.stream(o)) for o in range(prog.n_outputs))
    # several ragged inputs in one launch
    items = [data[:0], data[:5], data[: 70_001], data]
    many = prog.scan(pack_bytes(items), stats=True).stats
    assert many["tiles"] == prog.tiles_for([len(x) for x in items])
    for n, r in zip(many["tiles_run"], many["rows"]):
        assert r <= n <= min(many["tiles"], 32 * r)
    single = Program(groups, tuning=Tuning(prefilter=False))
    assert single.spec.n_parts == 0
    assert single.scan(inp, stats=True).stats == {"form": "single-kernel", "tiles": single.tiles_for([data.size])}


@pytest.mark.parametrize("every", [37, 400])
def test_text_dense_in_filter_keys(cuda, every):
    """Witnesses planted every `every` bytes put dozens of Bloom hits into each chunk of 32
    tiles; past the warp's record buffer a tile runs every term instead of looking its hits up.
    The split form is forced; streams equal the C oracle's."""
    from oracle import cpu
    ps = workloads.throughput_patterns(seed=3, n=64)
    groups = [compile_group(g) for g in ps.groups(4)]
    text = workloads.plant(workloads.printable_text(600_000, 61), ps.witnesses, every, 62)
    prog = Program(groups, tuning=Tuning(prefilter_limit=2.0))
    assert prog.spec.n_parts > 0
    res = prog.scan(pack_bytes([text]))
    want, counts = cpu.run_groups(groups, text)
    W = (text.size + 31) // 32
    for k, w in enumerate(want):
        assert first_diff(res.stream(k, 0).cpu().numpy(), w[:W]) is None, k
    assert res.counts[:, 0].tolist() == counts


@pytest.mark.parametrize("every", [4096, 64])
def test_more_than_1024_terms(cuda, every):
    """1024 regexes (more than 1024 terms, so more than 32 run-mask words per tile): every run
    word starts from the terms that always run and, past the record buffer, every word runs
    everything.  The scan is repeated over the same output and counts buffers, which must not
    change its result.  Streams equal the C oracle's."""
    from oracle import cpu
    ps = workloads.throughput_patterns(seed=83, n=1024)
    groups = [compile_group(g) for g in ps.groups(16)]
    text = workloads.plant(workloads.printable_text(300_000, 63), ps.witnesses, every, 64)
    prog = Program(groups)
    assert prog.spec.n_parts > 0 and prog.spec.n_run > 32
    inp = pack_bytes([text])
    want, counts = cpu.run_groups(groups, text)
    W = (text.size + 31) // 32
    for _ in range(2):
        res = prog.scan(inp)
        for k, w in enumerate(want):
            assert first_diff(res.stream(k, 0).cpu().numpy(), w[:W]) is None, k
        assert res.counts[:, 0].tolist() == counts


@pytest.mark.parametrize("single", [False, True])
def test_word_boundaries_and_case_flags(cuda, single):
    """Word boundaries (\\b, \\B: a look-ahead and a shift of the word class) and inline
    case-insensitive groups, in the split and the single-kernel form: streams and counts equal
    the C oracle's over text with planted witnesses, per regex and per group."""
    from oracle import cpu
    regexes = [r"\bhello\w+world\b", r"(?i)\bselect\s+\*\s+from\b", r"\Bing\b", r"\bzq\d{2,5}\b",
               r"(?i)passwd", r"x(?i:ab)y\B", r"\b[a-c]{3}\b", r"(?i)\bget /[a-z]+\.php"]
    wit = [b" helloXworld ", b" SeLeCt * FROM ", b"ringing ", b" zq123 ", b"PassWD", b"xABya",
           b" abc ", b" gEt /index.php"]
    groups = [compile_group(regexes[i::3]) for i in range(3)]
    text = workloads.plant(workloads.printable_text(250_000, 71), wit, 500, 72)
    prog = Program(groups, tuning=Tuning(prefilter=False) if single else Tuning(), per_regex=True)
    assert (prog.spec.n_parts == 0) == single
    res = prog.scan(pack_bytes([text]))
    want, counts = cpu.run_groups(groups, text, per_regex=True)
    W = (text.size + 31) // 32
    for k, w in enumerate(want):
        assert first_diff(res.stream(k, 0).cpu().numpy(), w[:W]) is None, k
    assert res.counts[:, 0].tolist() == counts
    assert min(counts) > 0


@pytest.mark.parametrize("single", [False, True])
def test_input_anchors_on_ragged_inputs(cuda, single):
    r"""\A, \z, \Z (an Advance and a Lookahead of the all-ones stream, i.e. the input's own first
    and last positions), also with pattern after $ and \Z, on one launch over many inputs of
    ragged lengths, some ending in LF: every input's streams and counts equal the C oracle's,
    split and single-kernel form."""
    regexes = [r"\A\w+", r"(?i)\Ahttp", r"\d\z", r"[a-z]\Z", r"(a|\A)b", r"\x{41}\x{42}\b",
               r"\A\n", r"z\Z", r"b$\na", r"[ab]\Z\n"]
    groups = [compile_group(regexes[i::2]) for i in range(2)]
    prog = Program(groups, tuning=Tuning(prefilter=False) if single else
                   Tuning(wpt=1, prefilter_limit=1.0), per_regex=True)
    assert (prog.spec.n_parts == 0) == single
    tile_chars = prog.spec.tile_words * 32
    lens = list(range(0, 40)) + [tile_chars + d for d in (-33, -1, 0, 1, 32)] + [3 * tile_chars + 7]
    rnd = np.random.default_rng(5)
    items = []
    for k, n in enumerate(lens):
        t = bytearray(rand_text(n, 300 + k, b"abzAB09 \nhtTP").tobytes())
        if n > 4 and k % 3 == 0:
            t[:4] = b"HtTp"
        if n and rnd.random() < 0.4:
            t[-1] = 0x0A
        items.append(np.frombuffer(bytes(t), np.uint8))
    check(prog, groups, items, per_regex=True)


@pytest.mark.parametrize("single", [False, True])
def test_group_stars_without_loops(cuda, single):
    """Stars over fixed-length groups, or unions of fixed-length branches, compile to MatchStar
    over the bytes their matches cover (no while loop), so they run fused; chains thousands of
    bytes long cross many tiles.
    Streams and counts equal the C oracle's per regex, split and single-kernel form."""
    regexes = ["q(rs)*t", "(ab)+c", "x(abc)*y", "(a[0-9]){2,}z", "(ab|cd)*e", "k(xy)*",
               "(?i)(gh)+i", "m(n(op){2})*w", "u(vw|xyz)*u", "(jk|lmn|o)+p"]
    groups = [compile_group(regexes[i::2]) for i in range(2)]
    prog = Program(groups, tuning=Tuning(prefilter=False) if single else
                   Tuning(wpt=1, prefilter_limit=1.0), per_regex=True)
    assert (prog.spec.n_parts == 0) == single
    wit = [b"q" + b"rs" * 3000 + b"t", b"ab" * 700 + b"c", b"xabcabcy", b"a1a2a3z",
           b"abcdcdabe" * 3, b"kxyxyxy" * 500, b"GhgHghi", b"mnopopnopopw", b"rsrst", b"qt",
           b"u" + b"vwxyz" * 900 + b"u", b"jkolmnojkp", b"lmnoooop"]
    text = workloads.plant(workloads.printable_text(200_000, 81), wit, 60, 82)
    items = [text, np.frombuffer(b"q" + b"rs" * 5000 + b"t", np.uint8),
             np.frombuffer(b"ab" * 4000, np.uint8), np.zeros(0, np.uint8)]
    check(prog, groups, items, per_regex=True)


@pytest.mark.parametrize("single", [False, True])
def test_lookarounds_on_ragged_inputs(cuda, single):
    """Lookahead (a Lookahead of the content's match ends) and lookbehind (an Advance of them),
    positive and negative, over many inputs of ragged lengths with planted witnesses: streams
    and counts equal the C oracle's per regex, split and single-kernel form."""
    regexes = [r"abcd(?=x)", r"qrst(?!u)", r"(?<=ab)cdqx", r"(?<!a)bcdq",
               r"(?<![0-9])12[0-9]{2}(?![0-9])", r"(?<=ab|c)dqrs", r"qrr(?=r)r+",
               r"(?<=[0-9])xabc(?=[0-9])"]
    wit = [b"abcdx", b"abcdy", b"qrstu", b"qrstv", b"abcdqx", b"zbcdq", b"abcdq", b"1234",
           b"012345", b"abdqrs", b"cdqrs", b"qrrrr", b"1xabc2", b"xabc2"]
    groups = [compile_group(regexes[i::2]) for i in range(2)]
    prog = Program(groups, tuning=Tuning(prefilter=False) if single else
                   Tuning(wpt=1, prefilter_limit=1.0), per_regex=True)
    assert (prog.spec.n_parts == 0) == single
    tile_chars = prog.spec.tile_words * 32
    lens = list(range(0, 40)) + [tile_chars + d for d in (-33, -1, 0, 1, 32)] + [5 * tile_chars + 3]
    rnd = np.random.default_rng(9)
    items = []
    for k, n in enumerate(lens):
        t = bytearray(rand_text(n, 700 + k, b"abcdqrx0129 \n").tobytes())
        for _ in range(n // 40):
            w = wit[rnd.integers(len(wit))]
            at = int(rnd.integers(0, max(1, n - len(w))))
            t[at:at + len(w)] = w[:n - at]
        items.append(np.frombuffer(bytes(t), np.uint8))
    check(prog, groups, items, per_regex=True)


@pytest.mark.parametrize("single", [False, True])
def test_wide_class_repeats(cuda, single):
    """Repeats of classes and of fixed-length groups with bounds of 16 and more, built by
    doubling (Advances of up to half the bound), over text with runs around the bounds: streams
    and counts equal the C oracle's per regex, split and single-kernel form."""
    regexes = ["abcd.{0,40}wxyz", "kq[a-z]{10,40}yy", "zq[0-9]{16}", "mnop[ab]{20,}st",
               "gh(ij){2,20}kl", "uv(wx|yz){16,}"]
    wit = [b"abcd" + b"." * k + b"wxyz" for k in (0, 39, 40, 41)] + \
          [b"kq" + b"r" * k + b"yy" for k in (9, 10, 40, 41)] + \
          [b"zq" + b"7" * k for k in (15, 16, 17)] + [b"mnop" + b"ab" * k + b"st" for k in (9, 10, 30)] + \
          [b"gh" + b"ij" * k + b"kl" for k in (1, 2, 20, 21)] + [b"uv" + b"wxyz" * k for k in (7, 8, 9, 40)]
    groups = [compile_group(regexes[i::2]) for i in range(2)]
    prog = Program(groups, tuning=Tuning(prefilter=False) if single else
                   Tuning(wpt=1, prefilter_limit=1.0), per_regex=True)
    assert (prog.spec.n_parts == 0) == single
    text = workloads.plant(workloads.printable_text(100_000, 91), wit, 40, 92)
    check(prog, groups, [text, np.frombuffer(b"".join(wit), np.uint8)], per_regex=True)


@pytest.mark.skipif(not os.environ.get("BG_FUZZ_GPU"), reason="set BG_FUZZ_GPU=<programs> to run")
@pytest.mark.parametrize("single", [False, True])
def test_random_regex_programs_match_c_oracle(cuda, single):
    """Seeded random regex groups over every emitter construct (as in the CPU differential
    test), each program in both kernel forms over text biased to the regexes' bytes: streams
    and counts equal the C oracle's per regex.  Programs that keep a while loop are skipped."""
    import random
    from bitgen_gb300.compiler import NotFusable
    from bitgen_gb300.regex import UnsupportedRegex, _matches_empty, parse_regex
    from tests.test_oracle import _fuzz_regex
    rnd = random.Random(33)
    for _ in range(int(os.environ["BG_FUZZ_GPU"])):
        rs = []
        while len(rs) < 8:
            r = "qz" + _fuzz_regex(rnd, 3) + "k"
            try:
                if not _matches_empty(parse_regex(r)):
                    compile_group([r])
                    rs.append(r)
            except UnsupportedRegex:
                pass
        groups = [compile_group(rs[i::2]) for i in range(2)]
        try:
            prog = Program(groups, tuning=Tuning(prefilter=False) if single else
                           Tuning(wpt=1, prefilter_limit=1.0), per_regex=True, executor="fused")
        except NotFusable:
            continue
        items = [rand_text(n, rnd.randrange(1 << 30), b"qzkabcx0 \nAB") for n in (0, 5, 3000, 70000)]
        check(prog, groups, items, per_regex=True)
        prog.close()
