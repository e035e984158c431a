"""CPU: the drop-in boundary accepts the instruction lists BitGen's pass pipeline emits.

``tests/golden/passes.json`` holds what the reference's ``run_passes`` (bitgen/from_icgrep.py:
124-166) made of parsed Pablo under the runner's pass flags with short_circuit 0/1 and
graph_break -1/0/1, dumped from the live objects by ``bitgen_gb300.refir`` (made by
``tests/golden/make_golden.py passes``).  Each list, converted by ``refir.group_from_ir``, must
compute the same match streams as the program before the passes: the group's regexes
compiled by this project, or, for the reference's fixture program, the parser's own IR.
"""

import json
import os

import numpy as np
import pytest

from bitgen_gb300 import refir, workloads
from bitgen_gb300.regex import compile_group
from oracle.pablo_ref import run_group

HERE = os.path.join(os.path.dirname(__file__), "golden")
CASES = json.load(open(os.path.join(HERE, "passes.json")))
PARSER = json.load(open(os.path.join(HERE, "parser.json")))


def _text(seed, regexes):
    t = workloads.printable_text(6000, seed)
    if regexes:
        wits = [s.encode() for s in regexes if s.isalnum()]
        return workloads.plant(t, wits or [b"x"], 300, seed)
    # the fixture program scans XML-ish text
    rng = np.random.default_rng(seed)
    alpha = np.frombuffer(b"<>/=\"' abcxyz\n?!-[]&;", np.uint8)
    return alpha[rng.integers(0, alpha.size, 6000)]


@pytest.mark.parametrize("case", sorted(CASES))
def test_pass_output_computes_the_same_streams(case):
    c = CASES[case]
    got = refir.group_from_ir(c["ir"])
    if c["regexes"]:
        want = compile_group(c["regexes"], matchstar=False)
    else:
        want = refir.group_from_ir(PARSER["reference_ir"]["xml_lexical_parsing"])
    for seed in (1, 2):
        text = _text(seed, c["regexes"])
        assert run_group(got, text) == run_group(want, text), (case, seed)


def test_every_flag_set_and_the_reference_fixture_are_covered():
    kinds = {k.split("/", 1)[1] for k in CASES}
    assert {"short_circuit=0/graph_break=-1", "short_circuit=1/graph_break=-1",
            "short_circuit=0/graph_break=0", "short_circuit=1/graph_break=1"} <= kinds
    assert any(k.startswith("xml_lexical_parsing/") for k in CASES)
    types = set()

    def walk(items):
        for it in items:
            types.add(it["type"])
            for key in ("body", "then", "else"):
                if it.get(key):
                    walk(it[key])
    for c in CASES.values():
        walk(c["ir"])
    # spills and reloads across graph breaks, their stream pointers, the kernel cuts, the
    # thread-bounds guard and the short-circuit jump text all occur
    assert {"STREAMSTORE", "STREAMLOAD", "STREAMDEFINE", "GRAPHBREAK", "IF", "STR", "WHILE"} <= types


def test_other_raw_cuda_text_is_rejected():
    ir = CASES["group0/short_circuit_text"]["ir"]
    bad = [dict(it) for it in ir]
    for it in bad:
        if it["type"] == "STR":
            it["text"] = "bs_adv = __funnelshift_r(a, b, 3);"
            break
    with pytest.raises(ValueError, match="raw CUDA text"):
        refir.group_from_ir(bad)
