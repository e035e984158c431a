"""Adapter from BitGen's bitstream IR (``bitgen/inst``) to this engine's Pablo IR.

BitGen's front end parses Pablo into ``BsInst`` lists (``bitgen/bitparser/bitstream_parser.py:
249-279``): eight ``STREAMLOAD`` of the basis planes, the program, and a final ``STREAMSTORE``
(``bs_result_stream |= <last result>``).  For the CUDA backend a ``SEL`` is already split into
NOT / AND / AND / OR (``bitstream_parser.py:214-227``).  These functions turn such a list, given
either as live objects with the parser's ``var_name_map`` or as the JSON form written by
``tests/golden/make_golden.py``, into a :class:`bitgen_gb300.pablo.Group`.  Only the IR's
meaning is used; performance passes that inject raw CUDA text (``BsStr`` from ``cc_advance`` /
``graph_break``) have no meaning here and are rejected.
"""

from __future__ import annotations

from typing import Dict, List

from .pablo import Group, If, Op, While

_BIN = {"AND": "and", "OR": "or", "XOR": "xor"}


def _convert(items, name, result_box) -> List:
    out: List = []
    for it in items:
        t = it["type"]
        ops = it.get("operands", [])
        ret = it.get("ret")
        if t == "STREAMLOAD":
            continue
        if t == "STREAMSTORE":
            result_box[0] = name(ops[0])
            continue
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
            out.append(While(name(it["cond"]), _convert(it["body"], name, result_box)))
        elif t == "IF":
            out.append(If(name(it["cond"]), _convert(it["then"], name, result_box),
                          _convert(it["else"], name, result_box) if it.get("else") is not None else None))
        else:
            raise ValueError(f"IR instruction {t} has no meaning for this engine")
    return out


def _name(v: str) -> str:
    return v if v != "output.matches" else "output_matches"


def group_from_ir(items: List[dict]) -> Group:
    """Group from the JSON dump of a reference instruction list."""
    box = [None]
    stmts = _convert(items, _name, box)
    if box[0] is None:
        last = [s for s in stmts if isinstance(s, Op)]
        box[0] = last[-1].dst
    return Group(stmts, box[0])


def _dump(inst, names: Dict[int, str]) -> dict:
    def nm(o):
        return names.get(o, str(o)) if isinstance(o, int) else str(o)

    t = inst.type.name
    d = {"type": t, "ret": nm(inst.ret) if not isinstance(inst.ret, list) else None}
    if t == "WHILE":
        d["cond"] = nm(inst.condition)
        d["body"] = [_dump(x, names) for x in inst.body.body]
    elif t == "IF":
        d["cond"] = nm(inst.condition)
        d["then"] = [_dump(x, names) for x in inst.body_1.body]
        d["else"] = [_dump(x, names) for x in inst.body_2.body] if inst.body_2 is not None else None
    elif t == "SEL":
        d["cond"] = nm(inst.condition)
        d["operands"] = [nm(o) for o in inst.operands]
    elif t == "STR":
        raise ValueError("raw CUDA text (cc_advance / graph_break passes) cannot be executed")
    else:
        d["operands"] = [nm(o) for o in inst.operands]
    return d


def group_from_bsinsts(insts, var_name_map: Dict[int, str]) -> Group:
    """Group from live ``BsInst`` objects and the parser's ``var_name_map``."""
    return group_from_ir([_dump(i, var_name_map) for i in insts])
