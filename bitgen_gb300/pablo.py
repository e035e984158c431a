"""Pablo bitstream programs: the IR the engine executes, and a parser for the text dialect.

The dialect is the one BitGen's front end reads (icgrep's ``-print-pablo`` output):

* ``x = (a & b)``, ``(a | b)``, ``(a ^ b)``, ``~a`` / ``(~a)``, ``(c ? a : b)``
  (``bitgen/bitparser/bitstream_parser.py:47-100``);
* ``x = pablo.Advance(a, n)``, ``pablo.MatchStar(m, c)``, ``pablo.ScanThru(m, c)``,
  ``pablo.Lookahead(a, n)`` (icgrep's later Pablo has it; the reference parser does not; used
  here for the ``$`` anchor)
  (``operation_name_map``, ``bitstream_parser.py:9-17``).  The reference parser raises
  ``NotImplementedError`` for the last two (``bitstream_parser.py:202-211``); this engine
  executes them;
* ``Next(x) = ...`` writes the loop-carried variable ``x`` (``bitstream_parser.py:68-69``);
* ``while v:`` / ``if v:`` / ``else:`` blocks delimited by indentation
  (``bitstream_parser.py:113-147``), with *whole-stream* conditions: the body of ``while v``
  runs again while any bit of ``v`` is set anywhere in the stream, as the reference's Python
  and torch lowerings state (``bitgen/inst/inst_block_while.py:137-153``,
  ``bitgen/inst/inst_block_if.py:314-342``);
* ``output.matches = x`` names the program's result.  Without it the result is the variable
  written by the last statement, as ``bitstream_parser.py:270-276`` stores ``insts[-1].ret``.

``basis0`` .. ``basis7`` are the transposed input planes (plane ``i`` holds bit ``7 - i`` of
every byte, ``bitgen/bitstream.py:228-258``); ``0`` and ``1`` are the all-zero and all-one
streams (``bitgen/inst/inst.py:66-69``).

The IR here is deliberately small: ``Op`` (one assignment), ``While`` and ``If``.  ``Group``
holds one regex group's program and, when the program came from the regex emitter in this
package, the per-regex result variables whose OR is the group result.
"""

from __future__ import annotations

import re
from dataclasses import dataclass, field
from typing import List, Optional, Sequence, Union

BASIS = tuple(f"basis{i}" for i in range(8))
CONSTS = ("0", "1")

# op name -> number of stream operands (Advance also carries an integer shift)
OP_ARITY = {
    "assign": 1,
    "not": 1,
    "and": 2,
    "or": 2,
    "xor": 2,
    "sel": 3,        # sel(c, a, b) = (c & a) | (~c & b)
    "advance": 1,    # advance(a; n)
    "lookahead": 1,  # lookahead(a; n): position p takes a[p + n]; zeros enter past the end
    "matchstar": 2,  # matchstar(m, c) = (((m & c) + c) ^ c) | m
    "scanthru": 2,   # scanthru(m, c) = (m + c) & ~c
}


@dataclass
class Op:
    dst: str
    op: str
    args: tuple
    shift: int = 0  # Advance distance

    def __post_init__(self):
        if self.op not in OP_ARITY:
            raise ValueError(f"unknown op {self.op}")
        if len(self.args) != OP_ARITY[self.op]:
            raise ValueError(f"{self.op} takes {OP_ARITY[self.op]} operands, got {self.args}")
        if self.op in ("advance", "lookahead") and self.shift < 0:
            raise ValueError("Advance / Lookahead distance must be >= 0")

    def text(self) -> str:
        a = self.args
        if self.op == "assign":
            rhs = a[0]
        elif self.op == "not":
            rhs = f"(~{a[0]})"
        elif self.op in ("and", "or", "xor"):
            sym = {"and": "&", "or": "|", "xor": "^"}[self.op]
            rhs = f"({a[0]} {sym} {a[1]})"
        elif self.op == "sel":
            rhs = f"({a[0]} ? {a[1]} : {a[2]})"
        elif self.op == "advance":
            rhs = f"pablo.Advance({a[0]}, {self.shift})"
        elif self.op == "lookahead":
            rhs = f"pablo.Lookahead({a[0]}, {self.shift})"
        elif self.op == "matchstar":
            rhs = f"pablo.MatchStar({a[0]}, {a[1]})"
        else:
            rhs = f"pablo.ScanThru({a[0]}, {a[1]})"
        return f"{self.dst} = {rhs}"


@dataclass
class While:
    cond: str
    body: List["Stmt"]


@dataclass
class If:
    cond: str
    then: List["Stmt"]
    orelse: Optional[List["Stmt"]] = None


Stmt = Union[Op, While, If]


@dataclass
class Group:
    """One regex group: a Pablo program whose result is ``result``.

    ``regex_results`` (optional) lists variables holding each member regex's own match
    stream; the group result is their OR.  ``regexes`` records the source patterns.
    """

    stmts: List[Stmt]
    result: str
    regex_results: Optional[List[str]] = None
    regexes: Optional[List[str]] = None

    def to_pablo(self) -> str:
        lines: List[str] = []

        def emit(stmts, ind):
            for s in stmts:
                if isinstance(s, Op):
                    lines.append(" " * ind + s.text())
                elif isinstance(s, While):
                    lines.append(" " * ind + f"while {s.cond}:")
                    emit(s.body, ind + 2)
                else:
                    lines.append(" " * ind + f"if {s.cond}:")
                    emit(s.then, ind + 2)
                    if s.orelse is not None:
                        lines.append(" " * ind + "else:")
                        emit(s.orelse, ind + 2)

        # a program ending in "result = x" stores x directly: the reference's alias removal
        # (bitgen/passes/remove_alias.py:10-52) drops such an assignment but leaves the store
        # "output.matches = result" reading the removed name
        stmts, res = list(self.stmts), self.result
        last = stmts[-1] if stmts else None
        if (isinstance(last, Op) and last.op == "assign" and last.dst == res
                and not any(res in (s.args if isinstance(s, Op) else (s.cond,))
                            for s in walk(stmts[:-1]))):
            stmts, res = stmts[:-1], last.args[0]
        emit(stmts, 0)
        lines.append(f"output.matches = {res}")
        return "\n".join(lines) + "\n"


def walk(stmts: Sequence[Stmt]):
    """Yield every statement, depth first, in program order."""
    for s in stmts:
        yield s
        if isinstance(s, While):
            yield from walk(s.body)
        elif isinstance(s, If):
            yield from walk(s.then)
            if s.orelse:
                yield from walk(s.orelse)


def has_control_flow(stmts: Sequence[Stmt]) -> bool:
    return any(not isinstance(s, Op) for s in walk(stmts))


# ----------------------------------------------------------------------------------------
# Parser
# ----------------------------------------------------------------------------------------

class PabloSyntaxError(ValueError):
    pass


_FUNC = re.compile(r"^([\w\.]+)\s*\(\s*(.*?)\s*\)$")
_IDENT = re.compile(r"^[A-Za-z_][\w\.]*$")


def _strip_parens(e: str) -> str:
    e = e.strip()
    if e.startswith("(") and e.endswith(")"):
        e = e[1:-1].strip()
    return e


def _operand(tok: str, defined: set, lineno: int) -> str:
    tok = tok.strip()
    if tok in CONSTS or tok in BASIS:
        return tok
    if not _IDENT.match(tok):
        raise PabloSyntaxError(f"line {lineno}: bad operand {tok!r}")
    if tok not in defined:
        raise PabloSyntaxError(f"line {lineno}: use of undefined variable {tok!r}")
    return tok


def _parse_rhs(dst: str, expr: str, defined: set, lineno: int) -> Op:
    e = _strip_parens(expr)
    m = _FUNC.match(e)
    if m:
        fn, argtxt = m.group(1), m.group(2)
        args = [a.strip() for a in argtxt.split(",")]
        if fn == "Next":
            return Op(dst, "assign", (_operand(args[0], defined, lineno),))
        if fn in ("pablo.Advance", "pablo.Lookahead"):
            if len(args) != 2:
                raise PabloSyntaxError(f"line {lineno}: {fn} takes 2 arguments")
            op = "advance" if fn == "pablo.Advance" else "lookahead"
            return Op(dst, op, (_operand(args[0], defined, lineno),), shift=int(args[1]))
        if fn in ("pablo.MatchStar", "pablo.ScanThru"):
            if len(args) != 2:
                raise PabloSyntaxError(f"line {lineno}: {fn} takes 2 arguments")
            op = "matchstar" if fn == "pablo.MatchStar" else "scanthru"
            return Op(dst, op, tuple(_operand(a, defined, lineno) for a in args))
        raise PabloSyntaxError(f"line {lineno}: invalid function call {fn}")
    toks = e.split()
    if len(toks) == 5 and toks[1] == "?" and toks[3] == ":":
        return Op(dst, "sel", tuple(_operand(t, defined, lineno) for t in (toks[0], toks[2], toks[4])))
    if len(toks) == 3 and toks[1] in ("&", "|", "^"):
        op = {"&": "and", "|": "or", "^": "xor"}[toks[1]]
        return Op(dst, op, (_operand(toks[0], defined, lineno), _operand(toks[2], defined, lineno)))
    if len(toks) == 2 and toks[0] == "~":
        return Op(dst, "not", (_operand(toks[1], defined, lineno),))
    if len(toks) == 1:
        t = toks[0]
        if t.startswith("~"):
            return Op(dst, "not", (_operand(_strip_parens(t[1:]), defined, lineno),))
        return Op(dst, "assign", (_operand(t, defined, lineno),))
    raise PabloSyntaxError(f"line {lineno}: invalid expression {expr!r}")


def parse_pablo(text: str) -> Group:
    """Parse Pablo text into a :class:`Group`.

    Raises :class:`PabloSyntaxError` on malformed input or use of an undefined variable,
    where the reference raises ``ValueError`` (``bitstream_parser.py:41-45,71,78,88,94``).
    """
    raw = text.split("\n")
    lines = []  # (indent, content, lineno)
    for i, ln in enumerate(raw, 1):
        c = ln.split("#", 1)[0].rstrip()
        if not c.strip():
            continue
        ind = len(c) - len(c.lstrip(" "))
        lines.append((ind, c.strip(), i))

    defined = set(BASIS) | set(CONSTS)
    result: List[Optional[str]] = [None]
    last_dst: List[Optional[str]] = [None]

    def block(pos: int, ind: int):
        out: List[Stmt] = []
        while pos < len(lines) and lines[pos][0] == ind:
            _, c, ln = lines[pos]
            if c.startswith("while ") or c.startswith("while\t"):
                cond = c[len("while"):].strip().rstrip(":").strip()
                cond = _operand(cond, defined, ln)
                if pos + 1 >= len(lines) or lines[pos + 1][0] <= ind:
                    raise PabloSyntaxError(f"line {ln}: empty while body")
                body, pos = block(pos + 1, lines[pos + 1][0])
                out.append(While(cond, body))
                continue
            if c.startswith("if ") or c.startswith("if\t"):
                cond = c[len("if"):].strip().rstrip(":").strip()
                cond = _operand(cond, defined, ln)
                if pos + 1 >= len(lines) or lines[pos + 1][0] <= ind:
                    raise PabloSyntaxError(f"line {ln}: empty if body")
                then, pos = block(pos + 1, lines[pos + 1][0])
                orelse = None
                if pos < len(lines) and lines[pos][0] == ind and lines[pos][1].rstrip(":").strip() == "else":
                    if pos + 1 >= len(lines) or lines[pos + 1][0] <= ind:
                        raise PabloSyntaxError(f"line {lines[pos][2]}: empty else body")
                    orelse, pos = block(pos + 1, lines[pos + 1][0])
                out.append(If(cond, then, orelse))
                continue
            if "=" not in c:
                raise PabloSyntaxError(f"line {ln}: expected an assignment: {c!r}")
            lhs, rhs = c.split("=", 1)
            lhs = _strip_parens(lhs.strip())
            m = _FUNC.match(lhs)
            if m and m.group(1) == "Next":
                lhs = m.group(2).strip()
            if lhs == "output.matches":
                src = _operand(_strip_parens(rhs), defined, ln)
                result[0] = src
                last_dst[0] = src
                pos += 1
                continue
            if not _IDENT.match(lhs) or lhs in BASIS or lhs in CONSTS:
                raise PabloSyntaxError(f"line {ln}: cannot assign to {lhs!r}")
            op = _parse_rhs(lhs, rhs, defined, ln)
            defined.add(lhs)
            out.append(op)
            last_dst[0] = lhs
            pos += 1
        return out, pos

    if not lines:
        raise PabloSyntaxError("empty program")
    stmts, pos = block(0, lines[0][0])
    if pos != len(lines):
        raise PabloSyntaxError(f"line {lines[pos][2]}: unexpected indentation")
    res = result[0] if result[0] is not None else last_dst[0]
    if res is None:
        raise PabloSyntaxError("program defines no result")
    return Group(stmts, res)


def parse_pablo_file(path: str) -> Group:
    with open(path, "r") as f:
        return parse_pablo(f.read())
