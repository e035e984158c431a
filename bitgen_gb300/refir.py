"""Adapter from BitGen's bitstream IR (``bitgen/inst``) to this engine's Pablo IR.

BitGen's front end parses Pablo into ``BsInst`` lists (``bitgen/bitparser/bitstream_parser.py:
249-279``): eight ``STREAMLOAD`` of the basis planes from ``basic_stream``, the program, and a
final ``STREAMSTORE`` into ``bs_result_stream``.  For the CUDA backend a ``SEL`` is already split
into NOT / AND / AND / OR (``bitstream_parser.py:214-227``).  ``run_passes``
(``bitgen/from_icgrep.py:124-166``) then rewrites the list for the reference's code generator;
these functions turn the result, given either as live objects with the parser's
``var_name_map`` or as the JSON form written by ``tests/golden/make_golden.py``, into a
:class:`bitgen_gb300.pablo.Group`.  Only the IR's meaning is kept:

* ``graph_break`` (``bitgen/passes/graph_break.py``) cuts the program into kernels: a value used
  past a cut is stored to a temporary stream (``STREAMSTORE`` into ``<var>_stream``, line 36)
  and loaded back (``STREAMLOAD``, line 117) - an assignment through that stream; inside a
  loop a carried value goes to ``<var>_stream_next``, swapped with ``<var>_stream`` after
  every iteration (lines 308-319);
  ``STREAMDEFINE`` (the stream's pointer, line 83) and ``GRAPHBREAK`` (the cut) carry no
  value.  Stores are wrapped in ``if (idx < n_unit_basic)`` (lines 179, 405), the kernel's
  bounds check on its thread index, which holds for every position of the stream.
* ``short_circuit`` (``bitgen/passes/short_circuit.py:263-361``) adds raw CUDA text: a jump
  ``if (block_all_zeros(x, &zero_flag)) { goto LABELn; }`` over an AND chain that is zero
  when ``x`` is zero, and the label ``LABELn:``.  It skips work whose result is zero anyway,
  so both are dropped.
* Other raw CUDA text (``cc_advance`` shifts) has no meaning here and is rejected.
"""

from __future__ import annotations

import re
from typing import Dict, List

from .pablo import Group, If, Op, While

_BIN = {"AND": "and", "OR": "or", "XOR": "xor"}
_THREAD_GUARD = "idx < n_unit_basic"
_BASIS = re.compile(r"^basis[0-7]$")
_SHORT_JUMP = re.compile(r"^\s*if \(block_all_zeros\(\w+, &zero_flag\)\) \{ goto LABEL\d+; \}\s*$")
_SHORT_LABEL = re.compile(r"^\s*LABEL\d+:\s*$")


def _convert(items, name, result_box) -> List:
    out: List = []
    for it in items:
        t = it["type"]
        ops = it.get("operands", [])
        ret = it.get("ret")
        if t in ("STREAMDEFINE", "GRAPHBREAK"):
            continue
        if t == "STREAMLOAD":
            # a value reloaded after a graph break; the basis planes never change, so their
            # reloads (from basic_stream or from a spill of their own) are identities
            if ops and ops[0] != "basic_stream" and not _BASIS.match(ret or ""):
                out.append(Op(name(ret), "assign", (name(ops[0]),)))
            continue
        if t == "STREAMSTORE":
            if ret in (None, "bs_result_stream"):
                result_box[0] = name(ops[0])
            else:                                    # spilled for a reload
                out.append(Op(name(ret), "assign", (name(ops[0]),)))
            continue
        if t == "STR":
            text = it.get("text", "")
            if _SHORT_JUMP.match(text) or _SHORT_LABEL.match(text):
                continue
            raise ValueError(f"raw CUDA text {text!r} has no meaning for this engine")
        if t in _BIN:
            out.append(Op(name(ret), _BIN[t], (name(ops[0]), name(ops[1]))))
        elif t == "NOT":
            out.append(Op(name(ret), "not", (name(ops[0]),)))
        elif t == "ASSIGN":
            out.append(Op(name(ret), "assign", (name(ops[0]),)))
        elif t == "ADVANCE":
            out.append(Op(name(ret), "advance", (name(ops[0]),), shift=int(ops[1])))
        elif t == "MATCHSTAR":
            out.append(Op(name(ret), "matchstar", (name(ops[0]), name(ops[1]))))
        elif t == "SCANTHRU":
            out.append(Op(name(ret), "scanthru", (name(ops[0]), name(ops[1]))))
        elif t == "SEL":
            out.append(Op(name(ret), "sel", (name(it["cond"]), name(ops[0]), name(ops[1]))))
        elif t == "WHILE":
            body = _convert(it["body"], name, result_box)
            # the loop swaps each double-buffered stream with its "_next" store after every
            # iteration (graph_break.py:308-319, inst_block_while.py:126)
            for cur, nxt in it.get("swap", []):
                body.append(Op(name(cur), "assign", (name(nxt),)))
            out.append(While(name(it["cond"]), body))
        elif t == "IF" and it["cond"] == _THREAD_GUARD:
            out.extend(_convert(it["then"], name, result_box))
            if it.get("else"):
                raise ValueError("a thread-bounds guard with an else branch")
        elif t == "IF":
            out.append(If(name(it["cond"]), _convert(it["then"], name, result_box),
                          _convert(it["else"], name, result_box) if it.get("else") is not None else None))
        else:
            raise ValueError(f"IR instruction {t} has no meaning for this engine")
    return out


def _name(v: str) -> str:
    return v if v != "output.matches" else "output_matches"


def _check_defined(stmts, defined: set):
    """Every variable is defined before it is read (loop bodies may read what a later
    iteration defines, as long as it is defined before the loop too)."""
    for s in stmts:
        if isinstance(s, Op):
            for a in s.args:
                if a not in defined and a not in ("0", "1") and not a.startswith("basis"):
                    raise ValueError(f"the IR reads {a!r}, which no earlier instruction defines "
                                     f"(an assignment the reference's alias removal dropped?)")
            defined.add(s.dst)
        elif isinstance(s, While):
            if s.cond not in defined:
                raise ValueError(f"the IR's loop tests {s.cond!r} before it is defined")
            _check_defined(s.body, defined)
        else:
            if s.cond not in defined:
                raise ValueError(f"the IR's branch tests {s.cond!r} before it is defined")
            _check_defined(s.then, defined)
            if s.orelse:
                _check_defined(s.orelse, defined)


def group_from_ir(items: List[dict]) -> Group:
    """Group from the JSON dump of a reference instruction list."""
    box = [None]
    stmts = _convert(items, _name, box)
    if box[0] is None:
        last = [s for s in stmts if isinstance(s, Op)]
        box[0] = last[-1].dst
    _check_defined(stmts, set())
    return Group(stmts, box[0])


def _dump(inst, names: Dict[int, str]) -> dict:
    def nm(o):
        return names.get(o, str(o)) if isinstance(o, int) else str(o)

    t = inst.type.name
    d = {"type": t, "ret": nm(inst.ret) if not isinstance(inst.ret, list) else None}
    if t == "WHILE":
        d["cond"] = nm(inst.condition)
        d["body"] = [_dump(x, names) for x in inst.body.body]
        swaps = [re.findall(r"&(\w+)", c) for c in getattr(inst, "cuda_swap_pointer", [])]
        if swaps:
            d["swap"] = swaps
    elif t == "IF":
        d["cond"] = nm(inst.condition)
        d["then"] = [_dump(x, names) for x in inst.body_1.body]
        d["else"] = [_dump(x, names) for x in inst.body_2.body] if inst.body_2 is not None else None
    elif t == "SEL":
        d["cond"] = nm(inst.condition)
        d["operands"] = [nm(o) for o in inst.operands]
    elif t == "STR":
        d["text"] = inst.str
    else:
        d["operands"] = [nm(o) for o in (inst.operands or [])]
    return d


def group_from_bsinsts(insts, var_name_map: Dict[int, str]) -> Group:
    """Group from live ``BsInst`` objects and the parser's ``var_name_map``."""
    return group_from_ir([_dump(i, var_name_map) for i in insts])
