"""Regex -> Pablo compiler (stands in for the icgrep ``-print-pablo`` step).

BitGen turns each regex group into Pablo text by running icgrep
(``bitgen/tool/pcre2pablo.py:33-48``: ``-print-pablo``, ``-disable-matchstar``,
``-if-insertion-gap=2147483647``, ``-disable-Unicode-linebreak``).  icgrep is an external fork
that is not part of the reference tree, so this module is the project's own emitter.  It emits
the same dialect (see :mod:`bitgen_gb300.pablo`) and can emit unbounded repetition either as
``pablo.MatchStar`` or as the ``while`` loop form icgrep produces under ``-disable-matchstar``.

Match convention (stated here because icgrep's is not pinned by the reference's tests): the
result stream of a regex has bit ``p`` set iff some non-empty match of the regex ends with the
byte at position ``p`` (its last byte), with matches allowed to start anywhere.  Line semantics
follow grep with LF-only line breaks (``-disable-Unicode-linebreak``): ``.`` and negated classes
do not match LF, ``^`` matches at position 0 and after every LF.  ``*?`` / ``+?`` / ``??`` (lazy)
have the same set of match ends as their greedy forms and are compiled alike.

Supported syntax: literals and escapes (``\\xHH``, ``\\x{HH}``, ``\\n \\r \\t \\f \\v \\e \\a``,
octal ``\\0oo`` / ``\\o{ooo}``, control ``\\cX``, escaped punctuation, ``\\Q...\\E`` quoting),
classes ``[...]`` / ``[^...]`` with ranges and ``\\d \\D \\w \\W \\s \\S \\h \\H``, ``.``, ``\\N``,
word boundaries ``\\b`` / ``\\B`` (``\\b`` is a backspace inside a class), ``^``, ``$``, ``\\A``,
``\\z``, ``\\Z``, ``\\K`` (no effect on match ends), ``\\R`` (a line break, CR LF as one), groups ``(...)`` / ``(?:...)`` / named
(``(?P<n>...)``, ``(?<n>...)``, ``(?'n'...)``), comments ``(?#...)``, lookahead ``(?=X)`` /
``(?!X)`` (X of fixed length) and lookbehind ``(?<=X)`` / ``(?<!X)`` (X bounded, not matching
the empty string), the flags ``i`` (ASCII case-insensitive), ``s`` (``.`` matches LF), ``x`` (white space and
``#`` comments outside classes ignored) and ``m`` (no effect: lines are always honoured) as ``(?flags)`` up to the end of the enclosing group or
``(?flags:...)``, with ``-`` to turn them off, alternation, ``* + ? {m} {m,} {m,n}`` (greedy or
lazy) and, over one class, possessive (``c*+ c++ c?+ c{m,n}+``, also as an atomic group
``(?>c*)``).
Zero-width assertions filter both markers (below): ``$`` keeps the last bytes followed by
an LF or the end, ``L & ~Lookahead(~LF, 1)``, and the next positions that hold an LF.

Compilation keeps two markers per regex state: ``L`` (positions of the last byte consumed) and
``P`` (positions where the next byte is to be matched, i.e. ``Advance(L, 1)`` plus any
zero-width starts).  A character class ``C`` maps ``(L, P)`` to ``(P & C, Advance(P & C, 1))``;
``C*`` maps it to ``(L | (MatchStar(P, C) & C), MatchStar(P, C))``.  Character classes are
compiled to a shared, reduced decision diagram over ``basis0`` (bit 7) .. ``basis7`` (bit 0).
"""

from __future__ import annotations

import re
from dataclasses import dataclass
from typing import Dict, List, Optional, Tuple

from .pablo import Group, Op, While

LF = 0x0A


class UnsupportedRegex(ValueError):
    pass


# ----------------------------------------------------------------------------------------
# AST
# ----------------------------------------------------------------------------------------

@dataclass(frozen=True)
class CC:
    bytes_: frozenset


@dataclass(frozen=True)
class Seq:
    items: tuple


@dataclass(frozen=True)
class Alt:
    items: tuple


@dataclass(frozen=True)
class Rep:
    item: object
    lo: int
    hi: Optional[int]  # None = unbounded


@dataclass(frozen=True)
class Start:
    pass


@dataclass(frozen=True)
class End:
    pass


@dataclass(frozen=True)
class TextStart:
    """``\\A``: the start of the input only."""


@dataclass(frozen=True)
class TextEnd:
    """``\\z`` (the end of the input), or ``\\Z`` with final_lf (also before a final LF)."""
    final_lf: bool = False


@dataclass(frozen=True)
class Look:
    """A lookaround: ``(?=X)`` / ``(?!X)`` (ahead) or ``(?<=X)`` / ``(?<!X)`` (behind, neg)."""
    item: object
    behind: bool = False
    neg: bool = False


@dataclass(frozen=True)
class WordB:
    """``\\b`` (or ``\\B`` with neg): a word/non-word transition between two bytes (the input's
    ends count as non-word)."""
    neg: bool = False


ALL_BYTES = frozenset(range(256))
DIGIT = frozenset(range(0x30, 0x3A))
WORD = frozenset(list(range(0x30, 0x3A)) + list(range(0x41, 0x5B)) + list(range(0x61, 0x7B)) + [0x5F])
SPACE = frozenset([0x20, 0x09, 0x0A, 0x0B, 0x0C, 0x0D])
DOT = ALL_BYTES - {LF}

_SIMPLE_ESC = {"n": 0x0A, "r": 0x0D, "t": 0x09, "f": 0x0C, "v": 0x0B, "e": 0x1B, "a": 0x07}
HSPACE = frozenset([0x09, 0x20, 0xA0])      # PCRE's \h on bytes
_CLASS_ESC = {"d": DIGIT, "D": ALL_BYTES - DIGIT, "w": WORD, "W": ALL_BYTES - WORD,
              "s": SPACE, "S": ALL_BYTES - SPACE, "h": HSPACE, "H": ALL_BYTES - HSPACE}


def _fold(bs) -> frozenset:
    """The byte set with both cases of every ASCII letter in it."""
    out = set(bs)
    for b in bs:
        if 0x41 <= b <= 0x5A or 0x61 <= b <= 0x7A:
            out.add(b ^ 0x20)
    return frozenset(out)


def _unquote(s: str) -> str:
    """The regex with every ``\\Q...\\E`` span (to ``\\E`` or the end) replaced by its characters
    escaped one by one, so that a quantifier after it applies to the last one, as in PCRE."""
    out, i = [], 0
    while i < len(s):
        if s[i] == "\\" and s.startswith("Q", i + 1):
            j = s.find("\\E", i + 2)
            end = len(s) if j < 0 else j
            for ch in s[i + 2:end]:
                if ord(ch) > 0xFF:
                    raise UnsupportedRegex("characters above 0xFF are not supported")
                out.append(ch if ch.isalnum() and ord(ch) < 0x80 else "\\x%02x" % ord(ch))
            i = end if j < 0 else j + 2
        elif s[i] == "\\":
            out.append(s[i:i + 2])
            i += 2
        else:
            out.append(s[i])
            i += 1
    return "".join(out)


class _Parser:
    def __init__(self, s: str):
        self.s = _unquote(s)
        self.i = 0
        self.icase = False    # (?i): ASCII letters match either case
        self.dotall = False   # (?s): '.' matches LF too
        self.extended = False  # (?x): white space and #-comments outside classes are ignored

    def peek(self):
        return self.s[self.i] if self.i < len(self.s) else None

    def take(self):
        c = self.s[self.i]
        self.i += 1
        return c

    def parse(self):
        node = self.alt()
        if self.i != len(self.s):
            raise UnsupportedRegex(f"unexpected {self.s[self.i]!r} at {self.i} in {self.s!r}")
        return node

    def _skip_x(self):
        """In (?x) mode, step over white space and comments (to the end of the line)."""
        while self.extended and self.i < len(self.s):
            c = self.s[self.i]
            if c in " \t\n\r\f\v":
                self.i += 1
            elif c == "#":
                j = self.s.find("\n", self.i)
                self.i = len(self.s) if j < 0 else j + 1
            else:
                return

    def alt(self):
        items = [self.seq()]
        self._skip_x()
        while self.peek() == "|":
            self.take()
            items.append(self.seq())
        return items[0] if len(items) == 1 else Alt(tuple(items))

    def seq(self):
        items = []
        self._skip_x()
        while self.peek() is not None and self.peek() not in "|)":
            a = self.atom()
            a = self.quant(a)
            items.append(a)
            self._skip_x()
        return Seq(tuple(items))

    def quant(self, a):
        zero_width = isinstance(a, (Start, End, WordB, TextStart, TextEnd, Look))
        while True:
            self._skip_x()
            c = self.peek()
            if zero_width and c is not None and (c in "*+?" or (c == "{" and self._is_counted())):
                raise UnsupportedRegex("a quantifier on an assertion")
            if c == "*":
                self.take(); a = Rep(a, 0, None)
            elif c == "+":
                self.take(); a = Rep(a, 1, None)
            elif c == "?":
                self.take(); a = Rep(a, 0, 1)
            elif c == "{" and self._is_counted():
                self.take()
                j = self.s.index("}", self.i)
                body = self.s[self.i:j]
                self.i = j + 1
                if "," in body:
                    lo_s, hi_s = body.split(",", 1)
                    lo = int(lo_s) if lo_s.strip() else 0
                    hi = int(hi_s) if hi_s.strip() else None
                else:
                    lo = hi = int(body)
                if hi is not None and hi < lo:
                    raise UnsupportedRegex(f"bad repeat {{{body}}}")
                a = Rep(a, lo, hi)
            else:
                return a
            # lazy suffix: same match-end set as greedy
            if self.peek() == "?":
                self.take()
            elif self.peek() == "+":
                self.take()
                a = _possessive(a)

    def _is_counted(self):
        j = self.s.find("}", self.i)
        if j < 0:
            return False
        return re.fullmatch(r"\d+(,\d*)?|,\d+", self.s[self.i + 1:j]) is not None

    def _flags(self):
        """Parse the letters of a `(?flags` group up to ':' or ')'; returns (icase, dotall,
        extended, end) with the flags as they hold inside and `end` the closing character."""
        icase, dotall, extended, on = self.icase, self.dotall, self.extended, True
        while True:
            c = self.peek()
            if c is None:
                raise UnsupportedRegex("unterminated group flags")
            self.take()
            if c in ":)":
                return icase, dotall, extended, c
            if c == "-":
                on = False
            elif c == "i":
                icase = on
            elif c == "s":
                dotall = on
            elif c == "x":
                extended = on
            elif c == "m":
                pass    # ^ and $ already hold at every line (grep line semantics)
            else:
                raise UnsupportedRegex(f"group flag {c!r} is not supported")

    def atom(self):
        c = self.take()
        if c == "(":
            saved = (self.icase, self.dotall, self.extended)
            if self.s.startswith("?:", self.i):
                self.i += 2
            elif self.peek() == "?" and self.i + 1 < len(self.s) and self.s[self.i + 1] in "imsx-":
                self.take()
                icase, dotall, extended, end = self._flags()
                if end == ")":
                    # (?flags): the flags hold to the end of the enclosing group
                    self.icase, self.dotall, self.extended = icase, dotall, extended
                    return Seq(())
                self.icase, self.dotall, self.extended = icase, dotall, extended
            elif self.s.startswith(("?=", "?!", "?<=", "?<!"), self.i):
                behind = self.s[self.i + 1] == "<"
                neg = self.s[self.i + (2 if behind else 1)] == "!"
                self.i += 3 if behind else 2
                node = self.alt()
                if self.peek() != ")":
                    raise UnsupportedRegex("missing )")
                self.take()
                self.icase, self.dotall, self.extended = saved
                return Look(node, behind, neg)
            elif self.s.startswith("?>", self.i):     # atomic group: a possessive class repeat
                self.i += 2
                node = self.alt()
                if self.peek() != ")":
                    raise UnsupportedRegex("missing )")
                self.take()
                self.icase, self.dotall, self.extended = saved
                while isinstance(node, Seq) and len(node.items) == 1:
                    node = node.items[0]
                if isinstance(node, CC):
                    return node
                if isinstance(node, Rep) and isinstance(node.item, CC):
                    return _possessive(node)
                raise UnsupportedRegex("atomic groups other than over one class (repeated or not)")
            elif self.s.startswith("?#", self.i):     # (?#comment)
                j = self.s.find(")", self.i)
                if j < 0:
                    raise UnsupportedRegex("unterminated comment")
                self.i = j + 1
                return Seq(())
            elif re.match(r"\?(P?<|')[A-Za-z_]\w*[>']", self.s[self.i:]):
                # named group (?P<name>...), (?<name>...), (?'name'...): a plain group
                self.i = self.s.index(">" if self.s[self.i + 1] in "P<" else "'", self.i + 3) + 1
            elif self.peek() == "?":
                raise UnsupportedRegex("group modifiers other than (?:, names, comments and flags "
                                       "are not supported")
            node = self.alt()
            if self.peek() != ")":
                raise UnsupportedRegex("missing )")
            self.take()
            self.icase, self.dotall, self.extended = saved
            return node
        if c == "[":
            return CC(self.cls())
        if c == ".":
            return CC(ALL_BYTES if self.dotall else DOT)
        if c == "^":
            return Start()
        if c == "$":
            return End()
        if c == "\\":
            if self.peek() in ("b", "B"):
                return WordB(neg=self.take() == "B")
            if self.peek() == "A":
                self.take()
                return TextStart()
            if self.peek() in ("z", "Z"):
                return TextEnd(final_lf=self.take() == "Z")
            if self.peek() == "R":          # \R: CR LF, or one of LF VT FF CR NEL alone (it never
                self.take()                 # gives back the LF of a CR LF): (?>\r\n|[...])
                crlf = Seq((CC(frozenset([0x0D])), CC(frozenset([LF]))))
                return Alt((crlf, Seq((Look(crlf, behind=False, neg=True),
                                       CC(frozenset([LF, 0x0B, 0x0C, 0x0D, 0x85]))))))
            if self.peek() == "K":          # \K: resets the reported start, so match ends stay
                self.take()
                return Seq(())
            if self.peek() == "N":          # any byte but LF
                self.take()
                return CC(DOT)
            e = self.escape()
            return CC(e) if isinstance(e, frozenset) else CC(self._lit(e))
        if c in "*+?":
            raise UnsupportedRegex(f"nothing to repeat at {self.i - 1}")
        b = c.encode("latin1")
        return CC(self._lit(b[0]))

    def _lit(self, b: int) -> frozenset:
        return _fold([b]) if self.icase else frozenset([b])

    def escape(self, in_class: bool = False):
        c = self.take()
        if c == "b" and in_class:
            return 0x08   # backspace inside a class, as in PCRE
        if c == "x":
            if self.peek() == "{":      # \x{H..}: one byte value
                j = self.s.find("}", self.i)
                h = self.s[self.i + 1:j] if j > 0 else ""
                if not h or not re.fullmatch(r"[0-9A-Fa-f]{1,2}", h):
                    raise UnsupportedRegex("bad \\x{} escape (one byte only)")
                self.i = j + 1
                return int(h, 16)
            h = self.s[self.i:self.i + 2]
            if len(h) != 2:
                raise UnsupportedRegex("bad \\x escape")
            self.i += 2
            return int(h, 16)
        if c in _SIMPLE_ESC:
            return _SIMPLE_ESC[c]
        if c == "0":                    # \0, \0o, \0oo: octal
            m = re.match(r"[0-7]{0,2}", self.s[self.i:])
            self.i += m.end()
            return int("0" + m.group(0), 8)
        if c == "o" and self.peek() == "{":
            j = self.s.find("}", self.i)
            o = self.s[self.i + 1:j] if j > 0 else ""
            if not re.fullmatch(r"[0-7]{1,3}", o) or int(o, 8) > 255:
                raise UnsupportedRegex("bad \\o{} escape (one byte only)")
            self.i = j + 1
            return int(o, 8)
        if c == "c":                    # \cX: control character X ^ 0x40 (X upper-cased)
            x = self.take()
            if x is None or not (0x20 <= ord(x) < 0x7F):
                raise UnsupportedRegex("bad \\c escape")
            return ord(x.upper()) ^ 0x40
        if c in _CLASS_ESC:
            return _CLASS_ESC[c]
        if c.isalnum():
            raise UnsupportedRegex(f"unsupported escape \\{c}")
        return c.encode("latin1")[0]

    def cls(self):
        neg = False
        if self.peek() == "^":
            self.take()
            neg = True
        items = set()
        first = True
        while True:
            c = self.peek()
            if c is None:
                raise UnsupportedRegex("unterminated class")
            if c == "]" and not first:
                self.take()
                break
            first = False
            self.take()
            if c == "\\":
                lo = self.escape(in_class=True)
            else:
                lo = c.encode("latin1")[0]
            if isinstance(lo, frozenset):
                items |= lo
                continue
            if self.peek() == "-" and self.i + 1 < len(self.s) and self.s[self.i + 1] != "]":
                self.take()
                h = self.take()
                hi = self.escape(in_class=True) if h == "\\" else h.encode("latin1")[0]
                if isinstance(hi, frozenset) or hi < lo:
                    raise UnsupportedRegex("bad class range")
                items |= set(range(lo, hi + 1))
            else:
                items.add(lo)
        s = _fold(items) if self.icase else frozenset(items)
        if neg:
            s = ALL_BYTES - s - {LF}
        return s


def parse_regex(s: str):
    return _Parser(s).parse()


# ----------------------------------------------------------------------------------------
# Pablo builder with hash-consing (CSE) and constant folding
# ----------------------------------------------------------------------------------------

class _Builder:
    def __init__(self):
        self.scopes: List[Tuple[List, Dict]] = [([], {})]  # (stmts, cse-table)
        self.n = 0
        self.cc_memo: Dict = {}
        self.top = False

    @property
    def stmts(self):
        return self.scopes[0][0]

    def fresh(self, stem="t"):
        self.n += 1
        return f"{stem}_{self.n}"

    def _lookup(self, key):
        for _, table in reversed(self.scopes):
            if key in table:
                return table[key]
        return None

    def emit(self, op, args, shift=0, stem="t", cse=True):
        key = (op, tuple(args), shift)
        if cse:
            hit = self._lookup(key)
            if hit is not None:
                return hit
        d = self.fresh(stem)
        # loop-invariant values (character classes, line starts) are hoisted to the top
        # level so that they stay defined after a loop whose body never ran
        scope = self.scopes[0] if self.top else self.scopes[-1]
        scope[0].append(Op(d, op, tuple(args), shift=shift))
        if cse:
            scope[1][key] = d
        return d

    def assign(self, dst, src):
        self.scopes[-1][0].append(Op(dst, "assign", (src,)))

    # folded constructors ---------------------------------------------------------------
    def AND(self, a, b):
        if a == "0" or b == "0":
            return "0"
        if a == "1":
            return b
        if b == "1" or a == b:
            return a
        a, b = sorted((a, b))
        return self.emit("and", (a, b))

    def OR(self, a, b):
        if a == "1" or b == "1":
            return "1"
        if a == "0":
            return b
        if b == "0" or a == b:
            return a
        a, b = sorted((a, b))
        return self.emit("or", (a, b))

    def NOT(self, a):
        if a == "0":
            return "1"
        if a == "1":
            return "0"
        return self.emit("not", (a,))

    def SEL(self, c, a, b):
        if a == b:
            return a
        if b == "0":
            return self.AND(c, a)
        if a == "0":
            return self.AND(self.NOT(c), b)
        if a == "1":
            return self.OR(c, b)
        if b == "1":
            return self.OR(self.NOT(c), a)
        return self.emit("sel", (c, a, b))

    def ADV(self, a, n=1):
        if a == "0" or n == 0:
            return a
        return self.emit("advance", (a,), shift=n)

    def MATCHSTAR(self, m, c):
        if m == "0":
            return "0"
        if c == "0":
            return m
        return self.emit("matchstar", (m, c))

    # character classes ---------------------------------------------------------------
    def cc(self, s: frozenset) -> str:
        saved, self.top = self.top, True
        try:
            return self._cc(s, 0)
        finally:
            self.top = saved

    def _cc(self, s: frozenset, level: int) -> str:
        """Decision diagram deciding bit `level` (basis7 = bit 0 first) of the byte; `s` holds
        the byte's remaining high bits (byte >> level).  Deciding the low bits first makes the
        shared sub-functions the high-bit prefixes (e.g. "011" of every lowercase letter)."""
        if not s:
            return "0"
        span = 1 << (8 - level)
        if len(s) == span:
            return "1"
        key = (level, s)
        hit = self.cc_memo.get(key)
        if hit is not None:
            return hit
        s1 = frozenset(x >> 1 for x in s if x & 1)
        s0 = frozenset(x >> 1 for x in s if not x & 1)
        f1 = self._cc(s1, level + 1)
        f0 = self._cc(s0, level + 1)
        r = self.SEL(f"basis{7 - level}", f1, f0)
        self.cc_memo[key] = r
        return r


# ----------------------------------------------------------------------------------------
# Regex -> Pablo
# ----------------------------------------------------------------------------------------

class _Compiler:
    """Compiles one regex AST into the shared builder.  State = (L, P-or-None)."""

    def __init__(self, b: _Builder, matchstar: bool):
        self.b = b
        self.use_matchstar = matchstar
        self._sol = None

    def P(self, st):
        L, P = st
        return P if P is not None else self.b.ADV(L, 1)

    def eol(self):
        """Positions followed by LF or by the end of the input: ~Lookahead(~LF, 1)."""
        if getattr(self, "_eol", None) is None:
            lf = self.b.cc(frozenset([LF]))
            saved, self.b.top = self.b.top, True
            nlf = self.b.NOT(lf)
            la = self.b.emit("lookahead", (nlf,), shift=1)
            self._eol = self.b.NOT(la)
            self.b.top = saved
        return self._eol

    def lookaround(self, node: "Look"):
        """(after, before) of a lookaround, like word_boundary's.  Behind: E = the ends of X's
        matches (starting anywhere), so X ends just before the next position q iff
        Advance(E, 1) holds at q, and just before position p + 1 iff E holds at p.  Ahead, for
        X of fixed length m: X starts at q iff Lookahead(E, m - 1) holds at q (G), and at
        p + 1 iff Lookahead(G, 1) holds at p.  Negation complements after the shift, so that the
        positions past the input's end count as no match.  X must be bounded (no ``*``, ``+``
        or open ``{m,}``) and, ahead, of fixed length."""
        b = self.b
        if not _bounded(node.item):
            raise UnsupportedRegex("lookaround content must be bounded")
        saved, b.top = b.top, True     # depends on the bytes only
        try:
            if node.behind:
                if _matches_empty(node.item):
                    raise UnsupportedRegex("lookbehind content that matches the empty string")
                E = self.run(node.item, ("0", "1"))[0]
                after, before = E, b.ADV(E, 1)
            else:
                U = _fixed_sets(node.item, assertions=True)
                if U is None or not U:
                    raise UnsupportedRegex("lookahead content must have a fixed, non-zero length")
                E = self.run(node.item, ("0", "1"))[0]
                G = b.emit("lookahead", (E,), shift=len(U) - 1) if len(U) > 1 else E
                after, before = b.emit("lookahead", (G,), shift=1), G
            if node.neg:
                after, before = b.NOT(after), b.NOT(before)
        finally:
            b.top = saved
        return after, before

    def word_boundary(self, neg: bool):
        """(after, before): bit p of `after` = a word/non-word transition between bytes p and
        p + 1, i.e. W ^ Lookahead(W, 1); bit q of `before` = one between bytes q - 1 and q,
        i.e. Advance(W, 1) ^ W (W = the word class; positions outside the input are non-word).
        With `neg`, the complements (\\B)."""
        key = "_wb_neg" if neg else "_wb"
        hit = getattr(self, key, None)
        if hit is None:
            w = self.b.cc(WORD)
            saved, self.b.top = self.b.top, True
            la = self.b.emit("lookahead", (w,), shift=1)
            after = self.b.emit("xor", tuple(sorted((w, la))))
            before = self.b.emit("xor", tuple(sorted((self.b.ADV(w, 1), w))))
            if neg:
                after, before = self.b.NOT(after), self.b.NOT(before)
            self.b.top = saved
            hit = (after, before)
            setattr(self, key, hit)
        return hit

    def text_start(self):
        """Position 0 only: ~Advance(1, 1)."""
        if getattr(self, "_sot", None) is None:
            saved, self.b.top = self.b.top, True
            self._sot = self.b.NOT(self.b.ADV("1", 1))
            self.b.top = saved
        return self._sot

    def text_end(self, final_lf: bool):
        """The last position, ~Lookahead(1, 1); with final_lf also the position before a final
        LF: last | Lookahead(LF & last, 1)."""
        key = "_eotz" if final_lf else "_eot"
        hit = getattr(self, key, None)
        if hit is None:
            saved, self.b.top = self.b.top, True
            last = self.b.NOT(self.b.emit("lookahead", ("1",), shift=1))
            hit = last
            if final_lf:
                lf = self.b.cc(frozenset([LF]))
                hit = self.b.OR(last, self.b.emit("lookahead", (self.b.AND(lf, last),), shift=1))
            self.b.top = saved
            setattr(self, key, hit)
        return hit

    def sol(self):
        if self._sol is None:
            lf = self.b.cc(frozenset([LF]))
            saved, self.b.top = self.b.top, True
            self._sol = self.b.NOT(self.b.ADV(self.b.NOT(lf), 1))
            self.b.top = saved
        return self._sol

    def run(self, node, st):
        b = self.b
        if isinstance(node, End):
            # after a last byte p: p + 1 is LF or the end; at a next position q: q is an LF
            return (b.AND(st[0], self.eol()), b.AND(self.P(st), self.b.cc(frozenset([LF]))))
        if isinstance(node, TextEnd):
            # at a next position q < n only \Z can hold: q is the last byte and an LF
            before = b.AND(b.cc(frozenset([LF])), self.text_end(False)) if node.final_lf else "0"
            return (b.AND(st[0], self.text_end(node.final_lf)), b.AND(self.P(st), before))
        if isinstance(node, TextStart):
            return ("0", b.AND(self.P(st), self.text_start()))
        if isinstance(node, CC):
            c = b.cc(node.bytes_)
            L = b.AND(self.P(st), c)
            return (L, None)
        if isinstance(node, Seq):
            for it in node.items:
                st = self.run(it, st)
            return st
        if isinstance(node, Alt):
            outs = [self.run(it, st) for it in node.items]
            L = "0"
            P = "0"
            for o in outs:
                L = b.OR(L, o[0])
                P = b.OR(P, self.P(o))
            return (L, P)
        if isinstance(node, Start):
            return ("0", b.AND(self.P(st), self.sol()))
        if isinstance(node, WordB):
            after, before = self.word_boundary(node.neg)
            return (b.AND(st[0], after), b.AND(self.P(st), before))
        if isinstance(node, Look):
            after, before = self.lookaround(node)
            return (b.AND(st[0], after), b.AND(self.P(st), before))
        if isinstance(node, Rep):
            return self.rep(node, st)
        raise UnsupportedRegex(str(node))

    def opt(self, node, st):
        o = self.run(node, st)
        return (self.b.OR(st[0], o[0]), self.b.OR(self.P(st), self.P(o)))

    def rep(self, node, st):
        b = self.b
        if node.lo >= WIDE_REPEAT or (node.hi or 0) >= WIDE_REPEAT:
            U = _fixed_sets(node.item)
            if U:
                return self._rep_fixed(node, st, len(U))
        for _ in range(node.lo):
            st = self.run(node.item, st)
        if node.hi is not None:
            for _ in range(node.hi - node.lo):
                st = self.opt(node.item, st)
            return st
        return self.star(node.item, st)

    def _rep_fixed(self, node, st, m):
        """``X{lo,hi}`` (hi None: ``X{lo,}``) for an item X of fixed length m and a wide count,
        in O(log) steps instead of one per count: B_k = k matches of X back to back ending at
        q (B_1 = X's match ends, B_{i+j} = B_i & Advance(B_j, i m)); the last bytes of k in
        [lo, hi] matches from a next position are V = Advance(P, lo m - 1) & B_lo, widened while
        fewer than hi by V |= Advance(V, s m) & B_s with s at most the count covered so far plus
        one (so no count is skipped)."""
        b = self.b
        saved, b.top = b.top, True      # X's match ends depend on the bytes only
        memo = {1: self.run(node.item, ("0", "1"))[0]}
        b.top = saved

        def B(k):
            if k not in memo:
                i = k // 2
                memo[k] = b.AND(B(i), b.ADV(B(k - i), i * m))
            return memo[k]

        def widen(V, d):       # V holds the runs of k matches: those of k .. k + d
            done = 0
            while done < d:
                step = min(done + 1, d - done)
                V = b.OR(V, b.AND(b.ADV(V, step * m), B(step)))
                done += step
            return V

        P = self.P(st)
        if node.lo == 0:        # then hi >= WIDE_REPEAT
            V = widen(b.AND(b.ADV(P, m - 1), B(1)), node.hi - 1)
            return (b.OR(st[0], V), b.OR(P, b.ADV(V, 1)))
        V = b.AND(b.ADV(P, node.lo * m - 1), B(node.lo))
        if node.hi is None:
            return self.star(node.item, (V, None))
        return (widen(V, node.hi - node.lo), None)

    def star(self, item, st):
        b = self.b
        P = self.P(st)
        if isinstance(item, CC):
            c = b.cc(item.bytes_)
            if self.use_matchstar:
                ms = b.MATCHSTAR(P, c)
            else:
                ms = self._star_loop_cc(P, c)
            return (b.OR(st[0], b.AND(ms, c)), ms)
        U = _fixed_sets(item) if self.use_matchstar else None
        if U is not None and len(U) == 1:
            return self.star(CC(U[0]), st)
        if U is not None and not _self_overlapping(U):
            return self._star_fixed(item, len(U), st)
        branches = _branches(item) if self.use_matchstar and U is None else None
        if branches and not _branches_overlap(branches):
            return self._star_disjoint(branches, st)
        # general star: while loop over the frontier of post-positions
        test = b.fresh("test")
        accum = b.fresh("accum")
        accL = b.fresh("accL")
        b.assign(test, P)
        b.assign(accum, P)
        b.assign(accL, "0")
        body: List = []
        b.scopes.append((body, {}))
        o = self.run(item, ("0", test))
        px = self.P(o)
        nacc = b.NOT(accum)
        new = b.AND(px, nacc)
        b.assign(accum, b.OR(accum, px) if px != "0" else accum)
        b.assign(accL, b.OR(accL, o[0]) if o[0] != "0" else accL)
        b.assign(test, new)
        b.scopes.pop()
        b.scopes[-1][0].append(While(test, body))
        return (b.OR(st[0], accL), accum)

    def _star_fixed(self, item, n, st):
        """``item*`` for an item of fixed length n whose matches cannot overlap (two can start
        less than n apart nowhere), without a loop.  E = the end positions of the item's matches,
        H = E | Advance(E, 1) | ... | Advance(E, n - 1) (the bytes they cover).  A chain of
        matches starting at a next-position p ends at q = p + n - 1, q + n, ...: since matches
        cannot overlap, the run of H from q holds exactly that chain, so its ends are
        MatchStar(Advance(P, n - 1) & E, H) & E, and the next-positions follow them."""
        b = self.b
        saved, b.top = b.top, True      # E and H depend on the bytes only
        E = self.run(item, ("0", "1"))[0]
        H = E
        for d in range(1, n):
            H = b.OR(H, b.ADV(E, d))
        b.top = saved
        ends = b.AND(b.MATCHSTAR(b.AND(b.ADV(self.P(st), n - 1), E), H), E)
        return (b.OR(st[0], ends), b.OR(self.P(st), b.ADV(ends, 1)))

    def _star_disjoint(self, branches, st):
        """``item*`` for an item that is a union of fixed-length branches of different lengths,
        no two of whose matches can overlap, without a loop.  Per branch b of length m: E_b =
        its match ends, S_b = Lookahead(E_b, m - 1) its starts, and it covers S_b | Advance(S_b,
        1) | ... | Advance(S_b, m - 1).  Matches that cannot overlap make every run of covered
        bytes one chain of touching matches, so from a start x the chain's bytes are
        R = MatchStar(P & S, covered), its ends R & E and its next positions R & Advance(E, 1)."""
        b = self.b
        saved, b.top = b.top, True      # the branches' streams depend on the bytes only
        S, E, H = "0", "0", "0"
        for U in branches:
            m = len(U)
            Eb = self.run(Seq(tuple(CC(u) for u in U)), ("0", "1"))[0]
            Sb = b.emit("lookahead", (Eb,), shift=m - 1) if m > 1 else Eb
            E, S, H = b.OR(E, Eb), b.OR(S, Sb), b.OR(H, Sb)
            for d in range(1, m):
                H = b.OR(H, b.ADV(Sb, d))
        b.top = saved
        R = b.MATCHSTAR(b.AND(self.P(st), S), H)
        return (b.OR(st[0], b.AND(R, E)), b.OR(self.P(st), b.AND(R, b.ADV(E, 1))))

    def _star_loop_cc(self, P, c):
        """icgrep's -disable-matchstar form of MatchStar(P, c)."""
        b = self.b
        test = b.fresh("test")
        accum = b.fresh("accum")
        b.assign(test, P)
        b.assign(accum, P)
        body: List = []
        b.scopes.append((body, {}))
        m1 = b.emit("and", (test, c), cse=False)
        adv = b.emit("advance", (m1,), shift=1, cse=False)
        nacc = b.emit("not", (accum,), cse=False)
        new = b.emit("and", (adv, nacc), cse=False)
        b.assign(accum, b.emit("or", (adv, accum), cse=False))
        b.assign(test, new)
        b.scopes.pop()
        b.scopes[-1][0].append(While(test, body))
        return accum


WIDE_REPEAT = 16   # repeats of fixed-length items with a bound from here on: O(log) steps


def _fixed_sets(node, assertions: bool = False) -> Optional[List[frozenset]]:
    """Per offset, the bytes a match of `node` can hold there, if every match of it has the same
    length and (unless `assertions`, which then count as length 0) it holds no zero-width
    assertion; else None."""
    if isinstance(node, CC):
        return [node.bytes_]
    if isinstance(node, Seq):
        out: List[frozenset] = []
        for it in node.items:
            u = _fixed_sets(it, assertions)
            if u is None:
                return None
            out += u
        return out
    if isinstance(node, Alt):
        us = [_fixed_sets(it, assertions) for it in node.items]
        if not us or any(u is None for u in us) or len({len(u) for u in us}) != 1:
            return None
        return [frozenset().union(*col) for col in zip(*us)]
    if isinstance(node, Rep) and node.hi == node.lo:
        u = _fixed_sets(node.item, assertions)
        return None if u is None else u * node.lo
    if assertions and isinstance(node, (Start, End, WordB, TextStart, TextEnd, Look)):
        return []
    return None


def _branches(node, cap: int = 16, max_len: int = 24) -> Optional[List[Tuple[frozenset, ...]]]:
    """The item as a list of distinct fixed-length branches (per-offset byte sets), if it is a
    finite union of at most `cap` of them, none empty or longer than `max_len`; else None."""
    def expand(n):
        if isinstance(n, CC):
            return [(n.bytes_,)]
        if isinstance(n, Seq):
            out = [()]
            for it in n.items:
                sub = expand(it)
                if sub is None:
                    return None
                out = [a + c for a in out for c in sub]
                if len(out) > cap:
                    return None
            return out
        if isinstance(n, Alt):
            out = []
            for it in n.items:
                sub = expand(it)
                if sub is None:
                    return None
                out += sub
            return out if len(out) <= cap else None
        if isinstance(n, Rep) and n.hi is not None:
            sub = expand(n.item)
            if sub is None:
                return None
            out, power = [], [()]
            for k in range(n.hi + 1):
                if k >= n.lo:
                    out += power
                power = [a + c for a in power for c in sub]
                if len(out) + len(power) > cap:
                    return None
            return out
        return None
    bs = expand(node)
    if bs is None:
        return None
    bs = sorted(set(bs), key=lambda u: (len(u), [sorted(x) for x in u]))
    if not bs or any(len(u) == 0 or len(u) > max_len for u in bs):
        return None
    return bs


def _branches_overlap(bs) -> bool:
    """Whether two matches of these branches could overlap: branch j starting d >= 0 bytes
    after branch i's start, inside it, with every shared offset's byte sets meeting (the same
    branch at d = 0 is the same match)."""
    for i, U in enumerate(bs):
        for j, V in enumerate(bs):
            for d in range(len(U)):
                if i == j and d == 0:
                    continue
                if all(U[t] & V[t - d] for t in range(d, min(len(U), d + len(V)))):
                    return True
    return False


def _possessive(node):
    """A possessive repeat of a class, as repeats and a negative lookahead that force it to
    take as much of the run as it may: ``c{m,}+`` = ``c{m,}(?!c)``, and ``c{m,n}+`` =
    ``c{n}|c{m,n-1}(?!c)`` (all n bytes when the run has them, else the whole run)."""
    if not (isinstance(node, Rep) and isinstance(node.item, CC)):
        raise UnsupportedRegex("possessive repeats of anything but one class")
    not_c = Look(node.item, behind=False, neg=True)
    if node.hi is None:
        return Seq((node, not_c))
    full = Rep(node.item, node.hi, node.hi)
    if node.hi == node.lo:
        return full
    return Alt((full, Seq((Rep(node.item, node.lo, node.hi - 1), not_c))))


def _bounded(node) -> bool:
    """No unbounded repetition inside."""
    if isinstance(node, Rep):
        return node.hi is not None and _bounded(node.item)
    if isinstance(node, (Seq, Alt)):
        return all(_bounded(it) for it in node.items)
    if isinstance(node, Look):
        return _bounded(node.item)
    return True


def _matches_empty(node) -> bool:
    """Whether the node can match the empty string (assertions count as empty)."""
    if isinstance(node, CC):
        return False
    if isinstance(node, Seq):
        return all(_matches_empty(it) for it in node.items)
    if isinstance(node, Alt):
        return any(_matches_empty(it) for it in node.items)
    if isinstance(node, Rep):
        return node.lo == 0 or _matches_empty(node.item)
    return True


def _self_overlapping(U: List[frozenset]) -> bool:
    """Whether two matches of a fixed-length item with per-offset byte sets U could start d < n
    positions apart (for every offset they share, the two sets meet)."""
    n = len(U)
    return n == 0 or any(all(U[j + d] & U[j] for j in range(n - d)) for d in range(1, n))


def compile_group(regexes: List[str], matchstar: bool = True) -> Group:
    """Compile a regex group to one Pablo program.

    The group result is the OR of the member regexes' match-end streams, the shape
    BitGen's CUDA backend produces per group (``bitgen/bitparser/bitstream_parser.py:270-276``).
    ``regex_results`` holds each member's own stream.
    """
    b = _Builder()
    results = []
    for r in regexes:
        ast = parse_regex(r)
        comp = _Compiler(b, matchstar)
        L, _ = comp.run(ast, ("0", "1"))
        results.append(L)
    acc = "0"
    for L in results:
        acc = b.OR(acc, L)
    res = acc
    # give the group result and every per-regex result a stable, distinct name
    names = []
    for i, L in enumerate(results):
        nm = f"re_{i}"
        b.scopes[0][0].append(Op(nm, "assign", (L,)))
        names.append(nm)
    b.scopes[0][0].append(Op("result", "assign", (res,)))
    return Group(b.stmts, "result", regex_results=names, regexes=list(regexes))


def compile_regex(regex: str, matchstar: bool = True) -> Group:
    return compile_group([regex], matchstar=matchstar)
