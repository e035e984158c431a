"""CPU tests: the oracle pinned to the reference's golden vectors, and the host-side compiler.

* transpose restatement == reference CPU transpose (bitgen/bitstream.py:228-258) on its vectors;
* Advance / add / MatchStar == the reference numpy templates (bitgen/template/template.py);
* this project's Pablo parser == the reference parser's IR (semantically, on random inputs);
* regex emitter == independent NFA == Python ``re`` on random inputs;
* C word-parallel oracle == big-integer oracle (block and whole-stream modes);
* while -> MatchStar conversion preserves results.
"""

import json
import os
import random
import re

import numpy as np
import pytest

from bitgen_gb300.compiler import convert_star_loops, fusable, generate_kernel, Tuning, NotFusable
from bitgen_gb300.engine import lower_interp
from bitgen_gb300.grouping import balance_regex_groups, group_regex_in_list, regex_custom_length
from bitgen_gb300.pablo import Op, While, parse_pablo, PabloSyntaxError
from bitgen_gb300.refir import group_from_ir
from bitgen_gb300.regex import UnsupportedRegex, compile_group, compile_regex
from oracle import cpu
from oracle.nfa_ref import group_match_ends, match_ends
from oracle.pablo_ref import (advance, int_to_words, matchstar, run_group, transpose_ref,
                              words_to_int)

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def bools_to_int(b):
    return int("".join("1" if x else "0" for x in reversed(list(b))) or "0", 2)


def test_transpose_matches_reference_vectors():
    g = np.load(os.path.join(GOLDEN, "transpose.npz"))
    n = 0
    for k in g.files:
        if not k.startswith("in"):
            continue
        src, want = g[k], g[k.replace("in", "out", 1)]
        rows = src if src.ndim == 2 else src[None]
        for m, row in enumerate(rows):
            assert np.array_equal(transpose_ref(row), want.reshape(-1, 8, want.shape[-1])[m]), k
            n += 1
    assert n >= 9


def test_word_layout_roundtrip():
    rng = np.random.default_rng(0)
    for W in (1, 2, 7, 33):
        w = rng.integers(0, 1 << 32, size=W, dtype=np.uint64).astype(np.uint32)
        assert np.array_equal(int_to_words(words_to_int(w), W), w)
    # position 0 is the MSB of word 0 in the reference layout
    assert int_to_words(1, 1)[0] == 0x80000000


def test_ops_match_reference_templates():
    g = np.load(os.path.join(GOLDEN, "ops.npz"))
    for i in range(12):
        m, c, k = g[f"m{i}"], g[f"c{i}"], int(g[f"k{i}"])
        n = m.size
        mask = (1 << n) - 1
        M, Cc = bools_to_int(m), bools_to_int(c)
        assert advance(M, k, mask) == bools_to_int(g[f"adv{i}"])
        assert (M + Cc) & mask == bools_to_int(g[f"add{i}"])
        assert matchstar(M, Cc, mask) == bools_to_int(g[f"ms{i}"])


def test_parser_agrees_with_reference_parser():
    gold = json.load(open(os.path.join(GOLDEN, "parser.json")))
    rng = np.random.default_rng(1)
    for name, ir in gold["reference_ir"].items():
        ref_group = group_from_ir(ir)
        if name in gold["emitted_pablo"]:
            mine = parse_pablo(gold["emitted_pablo"][name])
        else:
            mine = None
        for n in (1, 31, 64, 257):
            data = rng.integers(0, 256, size=n, dtype=np.uint8)
            if name == "xml_lexical_parsing":
                data = np.frombuffer(bytes(rng.choice(list(b"<>abAB "), size=n)), np.uint8)
            r = run_group(ref_group, data)
            if mine is not None:
                assert run_group(mine, data) == r, (name, n)


def test_parser_rejects_bad_programs():
    for bad in ("x = (a & b)\n", "x = pablo.Foo(basis0, 1)\n", "basis0 = basis1\n", "x = (basis0 & basis1\n  y = x\n"):
        with pytest.raises(PabloSyntaxError):
            parse_pablo(bad)


REGEXES = [r"abc", r"a[bc]+d", r"x.*y", r"(ab|cd)e", r"a{2,5}", r"[a-c]{3}", r"^ab", r"(^|xy)z",
           r"a(bc)*d", r"a\d+b", r"[^a]b", r"k.{2,4}m", r"(a|b)*c", r"\x61\x62", r"a+?b", r"q(rs)+t",
           r"[0-9]{0,2}z"]


@pytest.mark.parametrize("matchstar_form", [True, False])
def test_emitter_matches_nfa_and_python_re(matchstar_form):
    rnd = random.Random(7)
    for r in REGEXES:
        g = parse_pablo(compile_regex(r, matchstar=matchstar_form).to_pablo())
        pr = re.compile(r.replace("[^", "[^\\n").encode(), re.M)
        for _ in range(6):
            n = rnd.randint(0, 90)
            data = bytes(rnd.choice(b"abcdxyzkmqrst\n0123") for _ in range(n))
            want_re = 0
            for e in range(n):
                if any(pr.fullmatch(data, s, e + 1) for s in range(e + 1)):
                    want_re |= 1 << e
            assert run_group(g, data) == match_ends(r, data) == want_re, (r, data)


FLAG_REGEXES = [r"(?i)abc", r"(?i)a[b-d]+e", r"x(?i:yz)w", r"(?i)x(?-i:y)z", r"(?s)a.b",
                r"(?i)[^a]b", r"a(?s:.)c", r"(?i)\x41b", r"(?im)^ab", r"(?i:a|B)c",
                r"\bab", r"ab\b", r"\bx\w*\b", r"a\Bb", r"\B0", r"(a|\b)b", r"[\b-c]x",
                r"\b(?i:yz)\b", "(?x) a b | c d", "(?x)[ ]x # a comment\n y", r"a(?x: b c )d",
                r"(?ix) A \  B", r"\Aab", r"\A\w+", r"(?i)\Axy|z\z", r"b\z", r"\w\Z", r"(a|\A)b",
                r"\x{41}b", r"(?i)[\x{61}-c]\Z"]


@pytest.mark.parametrize("matchstar_form", [True, False])
def test_emitter_flags_match_nfa_and_python_re(matchstar_form):
    """Inline flags: i (ASCII case-insensitive), s (dot matches LF), m (no effect), global
    and scoped, word boundaries \\b \\B, input anchors \\A \\z \\Z and \\x{HH}, against the
    regex module on mixed-case text with line feeds, spaces and a backspace."""
    rx = pytest.importorskip("regex")
    rnd = random.Random(11)
    for r in FLAG_REGEXES:
        g = parse_pablo(compile_regex(r, matchstar=matchstar_form).to_pablo())
        # a match ending with byte e: the pattern as a (variable-length) look-behind at e + 1,
        # so that an assertion at its end still sees the byte after it (these patterns match
        # no empty string)
        flags = ""
        body = r.replace("[^", "[^\\n").replace(r"\A", r"(?<![\s\S])").replace(
            r"\z", r"(?![\s\S])").replace(r"\Z", r"(?=\n?(?![\s\S]))")
        body = re.sub(r"\\x\{(\w+)\}", lambda m: "\\x%02x" % int(m.group(1), 16), body)
        if body.startswith("(?") and body[2:body.index(")")].isalpha():
            flags, body = body[:body.index(")") + 1], body[body.index(")") + 1:]
        pr = rx.compile((flags + "(?<=" + body + ")").encode(), rx.M)
        for _ in range(6):
            n = rnd.randint(0, 90)
            data = bytes(rnd.choice(b"aAbBcCdDeExXyYzZwW\n0 _\x08") for _ in range(n))
            if rnd.random() < 0.3:
                data += b"\n"
            want_re = 0
            for e in range(n):
                if pr.match(data, e + 1):
                    want_re |= 1 << e
            assert run_group(g, data) == match_ends(r, data) == want_re, (r, data)


# PCRE syntax the emitter accepts, each with an equivalent the regex module reads
PCRE_EQUIV = [(r"(?P<n>ab)+c", r"(?:ab)+c"), (r"(?<n>x|y)z", r"(?:x|y)z"), (r"(?'n'q)r", r"qr"),
              (r"a(?#note)b", r"ab"), (r"\Qa.b\E+", r"a\.b+"), (r"x\Q(*)\E", r"x\(\*\)"),
              (r"(?i)\Qab\E", r"(?i)ab"), (r"\012a", r"\na"), (r"\0", r"\x00"),
              (r"\o{101}b", r"Ab"), (r"\cAx|\cz", r"\x01x|\x1a"), (r"[\cA-\cC]x", r"[\x01-\x03]x"),
              (r"\h+x", r"[ \t\xa0]+x"), (r"[\h\d]y", r"[ \t\xa0\d]y"), (r"a\H", r"a[^ \t\xa0]"),
              (r"a\N", r"a[^\n]"), (r"b\N+c", r"b[^\n]+c"),
              (r"a\R", r"a(?:\r\n|(?!\r\n)[\n\x0b\x0c\r\x85])"),
              (r"a\R\n", r"a(?:\r\n|(?!\r\n)[\n\x0b\x0c\r\x85])\n"),
              (r"\R+b", r"(?:\r\n|(?!\r\n)[\n\x0b\x0c\r\x85])+b")]


@pytest.mark.parametrize("matchstar_form", [True, False])
def test_emitter_pcre_syntax_matches_equivalents(matchstar_form):
    """Named groups, comments, \\Q...\\E, octal and control escapes, \\h \\H \\N, \\R (CR LF as one
    break, never given back): the emitter's streams equal the NFA's and the regex module's for
    an equivalent pattern."""
    rx = pytest.importorskip("regex")
    rnd = random.Random(12)
    alphabet = b"abcqrxyzAB.()*\n\t \x00\x01\x02\x03\x1a\xa0\r\r\x85"
    for ours, theirs in PCRE_EQUIV:
        g = parse_pablo(compile_regex(ours, matchstar=matchstar_form).to_pablo())
        pr = rx.compile(("(?<=" + theirs + ")").encode("latin1"), rx.M)
        for _ in range(6):
            n = rnd.randint(0, 80)
            data = bytes(rnd.choice(alphabet) for _ in range(n))
            want = 0
            for e in range(n):
                if pr.match(data, e + 1):
                    want |= 1 << e
            assert run_group(g, data) == match_ends(ours, data) == want, (ours, data)


LOOK_REGEXES = [r"a(?=b)", r"a(?!b)", r"(?<=a)b", r"(?<!a)b", r"x(?=y[a-c])", r"(?<=ab|c)d",
                r"(?<![0-9])[0-9]{2}(?![0-9])", r"q(?=r)r+", r"(?i)(?<=x)y", r"(?<=a.)b",
                r"(?<=[0-9])x(?=[0-9])", r"b(?!c)(?!a)", r"(?<=^a)b", r"a(?=b$)", r"(?<!\w)ab"]


@pytest.mark.parametrize("matchstar_form", [True, False])
def test_lookarounds_match_nfa_and_regex_module(matchstar_form):
    """Lookahead (fixed length) and lookbehind (bounded), positive and negative, at the start,
    middle and end of patterns: the emitter's streams equal the NFA's and the regex module's."""
    rx = pytest.importorskip("regex")
    rnd = random.Random(13)
    for r in LOOK_REGEXES:
        g = parse_pablo(compile_regex(r, matchstar=matchstar_form).to_pablo())
        pr = rx.compile(("(?<=" + r.replace("(?i)", "") + ")").encode(),
                        rx.M | (rx.I if "(?i)" in r else 0))
        for _ in range(8):
            n = rnd.randint(0, 70)
            data = bytes(rnd.choice(b"abcdqrxyXY0129 \n") for _ in range(n))
            want = 0
            for e in range(n):
                if pr.match(data, e + 1):
                    want |= 1 << e
            assert run_group(g, data) == match_ends(r, data) == want, (r, data)
    for r in (r"a(?=b*)", r"(?<=a*)b", r"(?<=a?)b", r"x(?=a|bc)"):
        with pytest.raises(UnsupportedRegex):
            compile_regex(r)


MID_ASSERTIONS = [r"a$\nb", r"a$", r"ab$|c", r"a\z", r"a$\n^b", r"a\Z\n", r"(?:a$\n)+b",
                  r"a$b", r"a\zb", r"[ab]$[\na]", r"a\Z"]


@pytest.mark.parametrize("matchstar_form", [True, False])
def test_end_assertions_inside_patterns(matchstar_form):
    """$, \\z and \\Z followed by more pattern (filtering the next positions as well as the last
    bytes) equal the NFA and the regex module; \\K leaves match ends unchanged."""
    rx = pytest.importorskip("regex")
    rnd = random.Random(14)
    for r in MID_ASSERTIONS:
        g = parse_pablo(compile_regex(r, matchstar=matchstar_form).to_pablo())
        body = r.replace(r"\z", r"(?![\s\S])").replace(r"\Z", r"(?=\n?(?![\s\S]))")
        pr = rx.compile(("(?<=" + body + ")").encode(), rx.M)
        for _ in range(10):
            n = rnd.randint(0, 40)
            data = bytes(rnd.choice(b"abab\n\nc") for _ in range(n))
            want = 0
            for e in range(n):
                if pr.match(data, e + 1):
                    want |= 1 << e
            assert run_group(g, data) == match_ends(r, data) == want, (r, data)
    data = b"xaby xay abyab"
    assert run_group(compile_regex(r"a\Kb"), data) == run_group(compile_regex("ab"), data) != 0


WIDE_REPEATS = ["a.{0,20}b", "x[a-z]{10,40}y", "q[0-9]{16}", "(?s)a.{17,30}", "z[ab]{0,16}",
                "c.{20,}d", "[ab]{16,}", "k[ab]{3,18}", "^.{16}$", "(?i)q{16,17}", "(ab){16}",
                "x(ab){2,20}y", "(abc){0,17}d", "(ab|cd){16,}e", "(aa){16,18}", "z(a[bc]){0,30}"]


def test_wide_class_repeats_match_nfa_and_regex_module():
    """Repeats of classes and fixed-length groups with a bound of 16 or more are built by
    doubling (O(log) steps): equal to the NFA and the regex module, at every count around the
    bounds and on random text."""
    rx = pytest.importorskip("regex")
    rnd = random.Random(15)
    for r in WIDE_REPEATS:
        g = compile_regex(r)
        assert len(g.stmts) < 80
        pr = rx.compile(("(?<=" + r.replace("(?i)", "").replace("(?s)", "") + ")").encode(),
                        rx.M | (rx.I if "(?i)" in r else 0) | (rx.S if "(?s)" in r else 0))
        texts = [bytes(rnd.choice(b"aabbbaq1xyzcdk\n") for _ in range(rnd.choice([0, 30, 90])))
                 for _ in range(12)]
        for k in range(0, 45):     # one run of k bytes (or pairs) between the literals
            for fill in (b"b", b"5", b"Q", b"ab", b"ac", b"cd", b"abc"):
                texts.append(r.encode()[:1].lstrip(b"^([(?") + fill * k + b"dbye")
        for data in texts:
            want = 0
            for e in range(len(data)):
                if pr.match(data, e + 1):
                    want |= 1 << e
            assert run_group(g, data) == match_ends(r, data) == want, (r, data)


def _forward_ends(rx, r, data):
    """Ends e of non-empty matches [s, e] of `r`, by forward matching forced to stop at e + 1
    (a look-behind wrapper would run possessive repeats backwards)."""
    out = 0
    for e in range(len(data)):
        pe = rx.compile(("(?:" + r + ")(?<=\\A[\\s\\S]{%d})" % (e + 1)).encode(), rx.M)
        if any(pe.match(data, s) for s in range(e + 1)):
            out |= 1 << e
    return out


def test_possessive_and_atomic_class_repeats():
    """c*+, c++, c?+, c{m,n}+ and (?>c*) etc. take as much of the run as they may (repeats and
    a negative lookahead of the class): equal to the NFA and to the regex module's forward
    matching."""
    rx = pytest.importorskip("regex")
    rnd = random.Random(16)
    for r in ["a*+a", "xa++b", "a?+a", "x(?>a*)b", "x(?>[ab]+)b", "[ab]*+c", r"\d++\d",
              "q(?>a)b", "a++", "(?i)x?+X", "a{1,3}+a", "xa{2,3}+", "a{2}+b", "x(?>a{0,2})a",
              "a{2,}+b"]:
        g = parse_pablo(compile_regex(r).to_pablo())
        for _ in range(25):
            data = bytes(rnd.choice(b"aabbxXqc019\n") for _ in range(rnd.randint(0, 20)))
            assert run_group(g, data) == match_ends(r, data) == _forward_ends(rx, r, data), (r, data)
    for r in ("(?>ab|a)c", "(ab)++", "(a|b)*+"):
        with pytest.raises(UnsupportedRegex):
            compile_regex(r)


# (regex, loop-free): stars over fixed-length items, or over unions of fixed-length branches,
# whose matches cannot overlap compile without a while loop; the others keep icgrep's loop form
GROUP_STARS = [("q(rs)*t", True), ("(ab)+c", True), ("x(abc)*y", True), ("(a[0-9]){2,}z", True),
               ("(ab|cd)*e", True), ("(?i)(ab)*c", True), ("z(ab)*", True), ("(a(bc){2})*x", True),
               ("(a\\d)*", True), ("(aa)*b", False), ("((ab){2})*c", False), ("(a.)*b", False),
               ("(ab|cde)*f", True), ("x(ab|cde)+y", True), ("(q|rst)*u", True), ("(a|bc)*d", True),
               ("z(ab|cde|fghi)*", True), ("(abc|d)+", True), ("(ab|abc)*d", False),
               ("(ab|b)*c", False), ("(x[0-9]{1,3})*y", False), ("(ab|ba)*c", False)]


@pytest.mark.parametrize("regex,loop_free", GROUP_STARS)
def test_group_stars_match_the_loop_form_and_nfa(regex, loop_free):
    """The loop-free star (MatchStar over the bytes the item's matches cover) equals the NFA,
    icgrep's while-loop form and the C evaluator, on text biased toward long chains."""
    g = compile_regex(regex)
    assert fusable(g) == loop_free
    loop = compile_regex(regex, matchstar=False)
    assert any(isinstance(st, While) for st in loop.stmts)
    rnd = random.Random(hash(regex) & 0xFFFF)
    chars = sorted(set(re.sub(r"[^a-z0-9]", "", regex.replace("\\d", "7")).encode()))
    for k in range(30):
        n = rnd.choice([0, 1, 5, 40, 200])
        alphabet = bytes(chars) + (b"AB\n." if k % 3 == 0 else b"")
        data = bytes(rnd.choice(alphabet) for _ in range(n))
        want = match_ends(regex, data)
        assert run_group(g, data) == want == run_group(loop, data), (regex, data)
        if n:
            st, cnt = cpu.run_groups([g], np.frombuffer(data, np.uint8))
            assert int(cnt[0]) == bin(want).count("1")


_FUZZ_ATOMS = ["a", "b", "c", "ab", ".", "[ab]", "[^a]", "\\d", "\\w", "\\s", "x", "[a-c]", "\\n"]


def _fuzz_regex(rnd, depth):
    """A random regex over the constructs the emitter accepts (seeded)."""
    k = rnd.random()
    if depth <= 0 or k < 0.35:
        return rnd.choice(_FUZZ_ATOMS)
    if k < 0.55:
        return _fuzz_regex(rnd, depth - 1) + _fuzz_regex(rnd, depth - 1)
    if k < 0.65:
        return "(?:" + _fuzz_regex(rnd, depth - 1) + "|" + _fuzz_regex(rnd, depth - 1) + ")"
    if k < 0.80:
        q = rnd.choice(["*", "+", "?", "{2}", "{1,3}", "{0,2}", "{2,}", "{16,18}", "{0,17}"])
        return "(?:" + _fuzz_regex(rnd, depth - 1) + ")" + q
    if k < 0.85:
        return rnd.choice(["^", "$", "\\b", "\\B"]) + _fuzz_regex(rnd, depth - 1)
    if k < 0.90:
        return _fuzz_regex(rnd, depth - 1) + rnd.choice(["(?=a)", "(?!b)", "(?=ab)", "(?=[ab]c)"])
    if k < 0.95:
        return rnd.choice(["(?<=a)", "(?<!b)", "(?<=ab|c)", "(?<![0-9])"]) + _fuzz_regex(rnd, depth - 1)
    return "(?i:" + _fuzz_regex(rnd, depth - 1) + ")"


@pytest.mark.parametrize("seed", [1, 2])
def test_random_regexes_match_nfa_and_regex_module(seed):
    """Differential test on seeded random regexes mixing every construct (groups, alternation,
    all quantifiers including wide ones, anchors, word boundaries, lookarounds, case groups):
    the emitter's streams (MatchStar and while-loop forms), the NFA, the C evaluator and the
    regex module agree.  Patterns that can match the empty string are skipped (the convention
    counts non-empty matches only)."""
    rx = pytest.importorskip("regex")
    from bitgen_gb300.regex import _matches_empty, parse_regex
    rnd = random.Random(seed)
    tested = 0
    while tested < 150:
        r = _fuzz_regex(rnd, 4)
        try:
            if _matches_empty(parse_regex(r)):
                continue
            g = compile_regex(r)
            loop = compile_regex(r, matchstar=False)
        except UnsupportedRegex:
            continue
        pr = rx.compile(("(?<=" + r.replace("[^", "[^\n") + ")").encode(), rx.M)
        tested += 1
        for _ in range(3):
            n = rnd.randint(1, 50)
            data = bytes(rnd.choice(b"aabbcx0 \nAB") for _ in range(n))
            want = 0
            for e in range(n):
                if pr.match(data, e + 1):
                    want |= 1 << e
            assert run_group(g, data) == run_group(loop, data) == match_ends(r, data) == want, (r, data)
            st, cnt = cpu.run_groups([g], np.frombuffer(data, np.uint8))
            assert int(cnt[0]) == bin(want).count("1"), (r, data)


def test_emitter_on_dna_motifs_matches_nfa_and_c_oracle():
    """The genomic motif grammar (IUPAC classes, gapped `.{lo,hi}` motifs) over DNA text with N
    runs, line feeds and planted motifs: emitter + big-int oracle == NFA == C evaluator."""
    from bitgen_gb300 import workloads
    ps = workloads.dna_motifs(24, seed=5)
    text = workloads.plant(workloads.dna_text(6000, seed=6), ps.witnesses, 400, 9)
    text[1000:1300] = ord("N")
    data = text.tobytes()
    groups = [compile_group(g) for g in ps.groups(3)]
    for g, rx in zip(groups, ps.groups(3)):
        want = run_group(g, text)
        assert want == group_match_ends(rx, data) != 0
        code, ns, outs = lower_interp([g])
        st, cnt = cpu.run_code(code, ns, outs, text, block_words=64)
        assert words_to_int(st[0]) == want and int(cnt[0]) == bin(want).count("1")


def test_emitter_rejects_unsupported():
    for r in ("a$+", "(?=x*)", r"a\b*", r"a\Z+", "(ab)++", "(?>ab|c)", "(?i", r"\x{100}", r"\101",
              r"(?<=a+)b", r"\o{400}", r"[\N]", "\\Q\u0100\\E", r"(?#open"):
        with pytest.raises(UnsupportedRegex):
            compile_regex(r)


def test_star_loops_become_matchstar():
    g = compile_group(["ab*c", "x[0-9]*y"], matchstar=False)
    assert any(isinstance(s, While) for s in g.stmts)
    conv = convert_star_loops(g.stmts)
    assert not any(isinstance(s, While) for s in conv)
    assert sum(isinstance(s, Op) and s.op == "matchstar" for s in conv) == 2
    assert fusable(g)
    rng = np.random.default_rng(3)
    for n in (0, 5, 300):
        data = np.frombuffer(bytes(rng.choice(list(b"abcxy0129"), size=n)), np.uint8) if n else np.zeros(0, np.uint8)
        g2 = type(g)(conv, g.result)
        assert run_group(g, data) == run_group(g2, data)
    # a loop over a group (not a single class) keeps its while form
    assert not fusable(compile_group(["q(rs)*t"], matchstar=False))


@pytest.mark.parametrize("block_words", [1, 3, 256])
def test_c_oracle_matches_bigint_oracle(block_words):
    rnd = random.Random(11)
    for ms in (True, False):
        for trial in range(12):
            n = rnd.randint(0, 900)
            data = np.frombuffer(bytes(rnd.choice(b"abcdxyzkmqrst\n01") for _ in range(n)), np.uint8)
            g = compile_group(rnd.sample(REGEXES, rnd.randint(1, 4)), matchstar=ms)
            code, ns, outs = lower_interp([g])
            s, c = cpu.run_code(code, ns, outs, data, block_words=block_words)
            ref = run_group(g, data)
            assert words_to_int(s[0]) == ref
            assert int(c[0]) == bin(ref).count("1")


def test_interp_lowering_reuses_slots():
    g = compile_group([f"ab{c}d[0-9]+e" for c in "ghijklmnopqrstuv"])
    code, n_slots, outs = lower_interp([g])
    n_vars = len({s.dst for s in g.stmts})
    assert n_slots < n_vars  # live ranges let slots be reused
    for ins in code:
        if ins[0] in (5, 11):  # Advance / Lookahead never in place
            assert ins[1] != ins[2]


def test_halo_grows_with_advance_depth():
    src = "a = (basis0 & basis1)\nb = pablo.Advance(a, 100)\noutput.matches = b\n"
    g = parse_pablo(src)
    assert generate_kernel([g], Tuning(wpt=1)).halo_lanes == 4   # ceil(100 / 32)
    assert generate_kernel([g], Tuning(wpt=4)).halo_lanes == 1
    src2 = src.replace("output.matches = b", "c = pablo.MatchStar(b, a)\noutput.matches = c")
    assert generate_kernel([parse_pablo(src2)], Tuning(wpt=1)).halo_lanes == 5
    deep = "a = (basis0 & basis1)\nb = pablo.Advance(a, 2000)\noutput.matches = b\n"
    with pytest.raises(NotFusable):
        generate_kernel([parse_pablo(deep)], Tuning(wpt=1))


def test_grouping_follows_reference_rule():
    rx = ["abc", r"\x41\x42", "[a-z]+q", "hello.*world", "x", "yy", "zzz[0-9]"]
    assert regex_custom_length(r"\x41[abc]d") == 3
    groups = balance_regex_groups(list(rx), 3)
    assert sorted(sum(groups, [])) == sorted(rx)
    loads = [sum(regex_custom_length(r) for r in g) for g in groups]
    assert max(loads) - min(loads) <= max(regex_custom_length(r) for r in rx)
    assert group_regex_in_list(rx[:2], 5) == [[r"\x41\x42"], ["abc"]]   # both length 3, stable
    assert group_regex_in_list(rx, 0) == [[r] for r in rx]


def test_result_bit_order_matches_reference_reader():
    """Position p of a stream is bit 31 - p % 32 of word p // 32, as the runner's result reader
    (bitgen/bitstream.py:27-73, golden vectors) sees it: the oracle's word conversion, the
    big-endian unpacking the GPU tests read outputs with, and the per-group counts of a
    [S, M, G, W] result."""
    z = np.load(os.path.join(GOLDEN, "bitstream.npz"))
    i = 0
    while f"w{i}" in z:
        words, pos = z[f"w{i}"], z[f"pos{i}"]
        x = words_to_int(words)
        assert [p for p in range(32 * words.size) if (x >> p) & 1] == pos.tolist()
        assert np.array_equal(np.nonzero(np.unpackbits(words.astype(">u4").view(np.uint8)))[0], pos)
        assert bin(x).count("1") == int(z[f"count{i}"]) and pos[0] == 0
        assert np.array_equal(int_to_words(x, words.size), words)
        i += 1
    assert i == 4
    res = z["res4"]
    per_group = [sum(bin(words_to_int(res[0, m, g])).count("1") for m in range(res.shape[1]))
                 for g in range(res.shape[2])]
    assert per_group == z["res4_count_array"].tolist()


def test_grouping_matches_reference_vectors():
    """Groups (and custom lengths) equal those of the reference entry script's own functions
    (scripts/run_bitgen.py:71-116, run by tests/golden/make_golden.py) on the README regexes,
    the synthetic workloads' sets and edge-case group counts."""
    with open(os.path.join(GOLDEN, "grouping.json")) as f:
        cases = json.load(f)["cases"]
    assert len(cases) >= 10
    for c in cases:
        assert [regex_custom_length(r) for r in c["regexes"]] == c["lengths"], c["set"]
        assert group_regex_in_list(c["regexes"], c["n_groups"]) == c["groups"], (c["set"], c["n_groups"])


def test_pcre_reader_matches_reference_vectors(tmp_path):
    """`read_regex_file` reads a /regex/flags file as bitgen/tool/pcre.py:5-27 does (golden
    vectors from that function): blank lines skipped, text between the first and last slash,
    lines without a leading slash pair rejected."""
    from bitgen_gb300.grouping import read_regex_file
    with open(os.path.join(GOLDEN, "grouping.json")) as f:
        pcre = json.load(f)["pcre"]
    path = tmp_path / "set.regex"
    path.write_text(pcre["text"])
    assert read_regex_file(str(path)) == pcre["regexes"]
    assert len(pcre["bad"]) == 4
    for bad in pcre["bad"]:
        path.write_text(bad + "\n")
        with pytest.raises(ValueError):
            read_regex_file(str(path))


def test_readme_known_answer_count_16():
    """The reference's only published known answer (README.md:124-142): 8 Snort regexes over the
    first 10 000 bytes of snort_10KB.input in 4 groups give count 16."""
    kat = np.load(os.path.join(GOLDEN, "readme_kat.npz"))
    rx = [str(r) for r in kat["regexes"]]
    groups = group_regex_in_list(rx, int(kat["n_groups"]))
    data = kat["input"]
    total = sum(bin(run_group(compile_group(g), data)).count("1") for g in groups)
    assert total == int(kat["expected_count"]) == 16
    nfa = sum(bin(__import__("oracle.nfa_ref", fromlist=["x"]).group_match_ends(g, data.tobytes())).count("1")
              for g in groups)
    assert nfa == 16
