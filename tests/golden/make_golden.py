"""Generate the golden vectors under tests/golden/ by running the reference's own Python code.

Run in a checkout where the reference BitGen tree is available (path in BITGEN_REF, default
/root/reference); it is imported read-only with stub modules for its optional dependencies
(pandas, colorlog, colorama, matplotlib, the compiled ``bitgen.cuda`` extension).  The GPU-less
parts of the reference are what pin the oracle:

* ``transpose.npz``  - ``transpose_bytestream_to_bitstream_py`` (bitgen/bitstream.py:228-258) on
  seeded random inputs, including all 256 byte values and ragged lengths;
* ``ops.npz``        - numpy stream templates ``bs_advance`` / ``bs_add`` / ``bs_match_star``
  (bitgen/template/template.py:63-103) on seeded random bool streams;
* ``readme_kat.npz`` - the reference's quick-start known answer (``README.md:124-142``): the 8
  regexes of ``datasets_small/snort_small.regex``, the first 10 000 bytes of
  ``datasets_small/snort_10KB.input``, 4 groups, published count 16;
* ``parser.json``    - the reference parser's instruction list (type, operands, result) for the
  hand-written fixture bitgen/bitparser/xml_lexical_parsing.pablo and for Pablo emitted by this
  project (while-loop form), to pin the dialect this project's parser accepts;
* ``bitstream.npz``  - ``Bitstream`` (bitgen/bitstream.py:27-73), the runner's result reader, on
  seeded uint32 streams: set-bit positions of 1-D streams and ``get_count_array`` of
  ``[S, M, G, W]`` results, to pin the bit order this project's outputs are read with;
* ``grouping.json``  - the reference entry script's regex grouping (``group_regex_in_list`` /
  ``balance_regex_groups`` / ``regex_custom_length``, scripts/run_bitgen.py:71-116) on the
  README regexes, the synthetic workloads' pattern sets and edge cases.  The script's module
  imports the GPU runner, so only those three function definitions are taken from its source
  and executed.

* ``passes.json``    - the reference's pass pipeline (``run_passes``) applied to parsed Pablo
  under several pass flags, dumped from the live objects by ``bitgen_gb300.refir``: the IR
  the drop-in boundary must accept (see ``passes`` below).

Usage:  python tests/golden/make_golden.py [grouping|passes]   (only grouping.json / passes.json)
"""

from __future__ import annotations

import json
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REF = os.environ.get("BITGEN_REF", "/root/reference")


def import_reference():
    import logging

    class _Formatter(logging.Formatter):   # colorlog.ColoredFormatter's stand-in
        def __init__(self, *a, **k):
            super().__init__()

    os.environ.setdefault("PYTHONDONTWRITEBYTECODE", "1")
    sys.dont_write_bytecode = True
    for name in ("pandas", "colorlog", "colorama", "matplotlib", "matplotlib.pyplot"):
        m = types.ModuleType(name)
        m.Fore = types.SimpleNamespace(RED="", GREEN="", YELLOW="", BLUE="", RESET="", CYAN="")
        m.Style = types.SimpleNamespace(RESET_ALL="", BRIGHT="")
        m.ColoredFormatter = _Formatter
        sys.modules.setdefault(name, m)
    cuda = types.ModuleType("bitgen.cuda")
    cuda.byte_stream_transpose = lambda *a, **k: None
    cuda.cub_exclusive_scan = lambda *a, **k: None
    sys.modules["bitgen.cuda"] = cuda
    sys.path.insert(0, REF)
    import bitgen.config as cfg  # noqa: E402
    cfg.set_config("backend", "cuda")
    return cfg


def reference_functions(rel: str, keep: set) -> dict:
    """Function definitions `keep` of the reference file `rel`, executed from its source (the
    files' own imports pull in the GPU runner)."""
    import ast
    import re
    path = os.path.join(REF, rel)
    with open(path) as f:
        tree = ast.parse(f.read(), path)
    mod = ast.Module([n for n in tree.body if isinstance(n, ast.FunctionDef) and n.name in keep],
                     type_ignores=[])
    ns = {"re": re}
    exec(compile(mod, path, "exec"), ns)
    assert keep <= set(ns)
    return ns


def reference_grouping():
    """The three grouping functions of scripts/run_bitgen.py and the PCRE file reader of
    bitgen/tool/pcre.py."""
    ns = reference_functions("scripts/run_bitgen.py",
                             {"regex_custom_length", "balance_regex_groups", "group_regex_in_list"})
    ns.update(reference_functions("bitgen/tool/pcre.py", {"read_regex_from_pcre_file"}))
    return ns


def write_grouping():
    ref = reference_grouping()
    sys.path.insert(0, REPO)
    from bitgen_gb300 import workloads
    readme = ref["read_regex_from_pcre_file"](os.path.join(REF, "datasets_small/snort_small.regex"))
    thr = list(workloads.throughput_patterns(seed=3, n=256).regexes)
    dna = list(workloads.dna_motifs(64, seed=5).regexes)
    hand = [r"\x41\x42", "abc", "[a-z]+q", "hello.*world", "x", "yy", "zzz[0-9]", r"[\x00-\x1f]z",
            "q[^a]{2,4}", r"\x2f\x2a.*\x2a\x2f"]
    cases = []
    for name, rx, ns in (("readme", readme, (4, 1, 0, 3, 20)), ("throughput", thr, (16, 3)),
                         ("dna", dna, (4,)), ("hand", hand, (3, 5, 1, 0, -1, 100))):
        for n in ns:
            groups = ref["group_regex_in_list"](list(rx), n, 1)
            cases.append({"set": name, "regexes": rx, "n_groups": n, "groups": groups,
                          "lengths": [ref["regex_custom_length"](r) for r in rx]})
    # the PCRE file reader on edge-case lines (blank lines, spaces, flags, inner slashes)
    import tempfile
    text = "/abc/\n\n   /a\\/b[/]c/i  \n/x//\n/p/q/r/sm\n\t/\\x2f\\x2a/\n"
    with tempfile.NamedTemporaryFile("w", suffix=".regex", delete=False) as f:
        f.write(text)
    pcre = {"text": text, "regexes": ref["read_regex_from_pcre_file"](f.name), "bad": []}
    for bad in ("abc", "/abc", "x/abc/", "/"):
        with open(f.name, "w") as g:
            g.write(bad + "\n")
        try:
            ref["read_regex_from_pcre_file"](f.name)
        except ValueError:
            pcre["bad"].append(bad)
    os.unlink(f.name)
    with open(os.path.join(HERE, "grouping.json"), "w") as f:
        json.dump({"cases": cases, "pcre": pcre}, f, indent=0)


def main():
    if sys.argv[1:] == ["grouping"]:
        write_grouping()
        print("grouping.json written to", HERE)
        return
    if sys.argv[1:] == ["passes"]:
        import tempfile
        cfg = import_reference()
        sys.path.insert(0, REPO)
        passes(cfg, tempfile.mkdtemp(prefix="bg_golden_"))
        print("passes.json written to", HERE)
        return
    write_grouping()
    cfg = import_reference()
    import torch
    from bitgen import bitstream as ref_bs
    from bitgen.template import template as ref_tpl
    from bitgen.bitparser import BitstreamParser

    # ---- transpose: the CPU path ends in .cuda(); keep the tensor on the host -------------
    torch.Tensor.cuda = lambda self, *a, **k: self
    rng = np.random.default_rng(20261203)
    cases = {}
    lens = [32, 64, 96, 320, 1024]
    for i, n in enumerate(lens):
        cases[f"in{i}"] = rng.integers(0, 256, size=n, dtype=np.uint8)
    cases["in_all256"] = np.arange(256, dtype=np.uint8).repeat(1)
    cases["in_multi"] = rng.integers(0, 256, size=(3, 128), dtype=np.uint8)
    out = {}
    for k, v in cases.items():
        arr = v if v.ndim == 2 else v[None, :]
        t = torch.from_numpy(arr.copy())[None]           # [S=1, M, n]
        planes = ref_bs.transpose_bytestream_to_bitstream_py(t).numpy()
        out[k] = v
        out[k.replace("in", "out", 1)] = planes.astype(np.uint32)
    np.savez_compressed(os.path.join(HERE, "transpose.npz"), **out)

    # ---- numpy op templates ------------------------------------------------------------
    ops = {}
    for i in range(12):
        n = int(rng.integers(1, 300))
        dens = [0.05, 0.5, 0.95][i % 3]
        m = rng.random(n) < dens * 0.2
        c = rng.random(n) < dens
        k = int(rng.integers(1, 70))
        ops[f"m{i}"] = m
        ops[f"c{i}"] = c
        ops[f"k{i}"] = np.int64(k)
        ops[f"adv{i}"] = ref_tpl.bs_advance(m.copy(), k) if k < n else np.zeros(n, bool)
        ops[f"add{i}"] = ref_tpl.bs_add(m.copy(), c.copy())
        ops[f"ms{i}"] = ref_tpl.bs_match_star(m.copy(), c.copy())
    np.savez_compressed(os.path.join(HERE, "ops.npz"), **ops)

    # ---- result reader -------------------------------------------------------------------
    bsv = {}
    for i, W in enumerate((1, 2, 7, 33)):
        words = rng.integers(0, 1 << 32, size=W, dtype=np.uint64).astype(np.uint32)
        words[0] |= 1 << 31            # position 0 set
        bsv[f"w{i}"] = words.copy()
        pos = ref_bs.Bitstream(words.copy()).get_ones_pos()
        bsv[f"pos{i}"] = np.asarray(pos, dtype=np.int64)
        bsv[f"count{i}"] = np.int64(ref_bs.Bitstream(words.copy()).get_count())
    res4 = rng.integers(0, 1 << 32, size=(1, 2, 3, 5), dtype=np.uint64).astype(np.uint32)
    bsv["res4"] = res4.copy()
    bsv["res4_count_array"] = np.asarray(ref_bs.Bitstream(res4.copy()).get_count_array(), np.int64)
    np.savez_compressed(os.path.join(HERE, "bitstream.npz"), **bsv)

    # ---- README quick-start known answer ----------------------------------------------
    from bitgen.tool.pcre import read_regex_from_pcre_file
    rx = read_regex_from_pcre_file(os.path.join(REF, "datasets_small/snort_small.regex"))
    with open(os.path.join(REF, "datasets_small/snort_10KB.input"), "rb") as f:
        kat_input = np.frombuffer(f.read()[:10000], dtype=np.uint8)
    np.savez_compressed(os.path.join(HERE, "readme_kat.npz"), input=kat_input,
                        regexes=np.array(rx), n_groups=np.int64(4),
                        expected_count=np.int64(16))  # README.md:138-142 "count 16"

    # ---- parser ------------------------------------------------------------------------
    sys.path.insert(0, REPO)
    from bitgen_gb300.regex import compile_group

    def dump(path):
        p = BitstreamParser()
        insts = p.parse_file(path)
        names = p.var_name_map

        def enc(inst):
            d = {"type": inst.type.name, "ret": names.get(inst.ret, str(inst.ret))
                 if not isinstance(inst.ret, list) else [names.get(r, r) for r in inst.ret]}
            if inst.type.name == "WHILE":
                d["cond"] = names[inst.condition]
                d["body"] = [enc(x) for x in inst.body.body]
            else:
                ops_ = []
                for o in inst.operands:
                    ops_.append(names.get(o, o) if isinstance(o, int) else str(o))
                d["operands"] = ops_
            return d

        return [enc(x) for x in insts]

    parser_cases = {"xml_lexical_parsing": os.path.join(REF, "bitgen/bitparser/xml_lexical_parsing.pablo")}
    emitted = {}
    import tempfile
    tmpdir = tempfile.mkdtemp(prefix="bg_golden_")
    for name, rx in {"literal": ["abc"], "class_star": ["a[bc]*d"], "group_star": ["q(rs)*t"],
                     "alt": ["(ab|cd)e", "x{2,3}y"]}.items():
        g = compile_group(rx, matchstar=False)
        txt = g.to_pablo()
        path = os.path.join(tmpdir, f"golden_{name}.pablo")
        with open(path, "w") as f:
            f.write(txt)
        parser_cases[name] = path
        emitted[name] = txt
    res = {k: dump(v) for k, v in parser_cases.items()}
    with open(os.path.join(HERE, "parser.json"), "w") as f:
        json.dump({"reference_ir": res, "emitted_pablo": emitted}, f, indent=1, sort_keys=True)
    passes(cfg, tmpdir)
    print("golden vectors written to", HERE)


def passes(cfg, tmpdir):
    """passes.json: the instruction lists the reference's run_passes (bitgen/from_icgrep.py:
    124-166) makes of parsed Pablo, dumped from the live objects by this project's adapter
    (bitgen_gb300.refir._dump), under the runner's pass flags (scripts/run_bitgen.py:415-480
    defaults) with pass_cc_advanced = 0 and short_circuit / graph_break varied.

    The short-circuit pass finds no AND chain it rewrites in Pablo from this project's emitter
    (its chain search, short_circuit.py:91-130, expects icgrep's program shape), so the case
    "short_circuit_text" adds, in the pass's own form (BsStr, short_circuit.py:280-282 and
    352-353), a jump over an AND chain and its label: the adapter must drop both."""
    from bitgen import from_icgrep
    from bitgen.bitparser.bitstream_parser import BitstreamParser
    from bitgen.inst.inst import BsInstType
    from bitgen.inst.inst_str import BsStr
    from bitgen_gb300 import refir, workloads
    from bitgen_gb300.regex import compile_group

    defaults = {"pass_cc_advanced": 0, "pass_cc_advanced_max": 1, "pass_cc_advanced_merge_cc": 1,
                "pass_short_circuit_start": 2, "pass_short_circuit_interval": 2,
                "pass_short_circuit_interval_disable": 0, "pass_short_circuit_syncpoint": 1,
                "pass_print_graph": 0, "pass_inst_stats": 0, "pass_inst_stats_dyn": 0}
    for k, v in defaults.items():
        cfg.set_config(k, v)
    regexes = workloads.throughput_patterns(seed=3, n=8).regexes
    programs = {}
    for gi, g in enumerate(workloads.PatternSet(regexes, []).groups(2)):
        path = os.path.join(tmpdir, f"passes_{gi}.pablo")
        with open(path, "w") as f:
            f.write(compile_group(g, matchstar=False).to_pablo())
        programs[f"group{gi}"] = (path, g)
    programs["xml_lexical_parsing"] = (os.path.join(REF, "bitgen/bitparser/xml_lexical_parsing.pablo"), None)
    cases = {}
    for pname, (path, rx) in programs.items():
        for sc, gb in ((0, -1), (1, -1), (0, 0), (1, 0), (1, 1)):
            cfg.set_config("pass_short_circuit", sc)
            cfg.set_config("pass_graph_break", gb)
            p = BitstreamParser()
            insts = from_icgrep.run_passes(p.parse_file(path), p.var_name_map)
            cases[f"{pname}/short_circuit={sc}/graph_break={gb}"] = {
                "regexes": rx, "ir": [refir._dump(i, p.var_name_map) for i in insts]}
    # the pass's jump and label around the first AND chain after the first Advance
    cfg.set_config("pass_short_circuit", 1)
    cfg.set_config("pass_graph_break", -1)
    path, rx = programs["group0"]
    p = BitstreamParser()
    insts = from_icgrep.run_passes(p.parse_file(path), p.var_name_map)
    first_adv = next(i for i, x in enumerate(insts) if x.type == BsInstType.ADVANCE)
    at = next(i for i in range(first_adv, len(insts)) if insts[i].type == BsInstType.AND)
    end = next(i for i in range(at + 1, len(insts)) if insts[i].type != BsInstType.AND)
    var = p.var_name_map[insts[at].ret]
    insts = (insts[:at + 1]
             + [BsStr([f"if (block_all_zeros({var}, &zero_flag)) {{ goto LABEL0; }}"])]
             + insts[at + 1:end] + [BsStr(["LABEL0:"])] + insts[end:])
    cases["group0/short_circuit_text"] = {"regexes": rx,
                                          "ir": [refir._dump(i, p.var_name_map) for i in insts]}
    with open(os.path.join(HERE, "passes.json"), "w") as f:
        json.dump(cases, f, separators=(",", ":"), sort_keys=True)


if __name__ == "__main__":
    main()
