"""Compile Pablo groups into one fused sm_103a scan kernel (CUDA C++ for NVRTC).

This replaces what BitGen's CUDA code generator emits (``bitgen/codegen/gen_cuda.py:133-497``:
one ``regex_<g>`` device function per group, walked serially over the whole input by one CTA
per group, ``KernelGenerated`` dispatching on ``blockIdx.x``).  Here every group of the pattern
set is lowered into a single straight-line program that a warp runs on one tile of the input,
with all groups interleaved, so the input is read and transposed once (not once per group).

Pipeline
1. ``while`` loops in the form icgrep emits for an unbounded repetition of one character class
   under ``-disable-matchstar`` (``test = accum = P; while test: m = test & C;
   a = Advance(m, 1); test = a & ~accum; accum = accum | a``) are replaced by
   ``accum = MatchStar(P, C)``; both compute the positions reachable from ``P`` through runs
   of ``C``.  Programs that keep other loops or ``if`` blocks are not fusable (see
   :func:`fusable`) and run on the whole-stream executor.
2. Each group becomes SSA nodes; all groups share one hash-consed DAG.
3. Depth analysis: ``dbits(v)`` is how far (in characters) before a position ``v`` depends on.
   Advance adds its distance; an addition is exact one lane after its inputs are exact.  The
   halo ``HL`` (lanes) covers the deepest output, so lanes ``[HL, 32)`` of a tile are exact.
4. Code generation with zero-block skipping: a chain of zero-preserving steps (``AND``,
   ``Advance``) is emitted inside ``if (bg::any(x))`` blocks, so the rest of a regex is skipped
   for a whole warp tile as soon as its marker is zero, the semantics of the reference's
   short-circuit pass (``bitgen/passes/short_circuit.py:91-388``).  Character classes are
   re-materialised inside the blocks that use them.  Additions always run (their carry may
   arrive from the previous tile) and take their marker as zero when its chain was skipped.
"""

from __future__ import annotations

import hashlib
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence, Tuple

from .pablo import BASIS, Group, If, Op, While, walk

CHAIN_OPS = ("and", "advance")
ADD_OPS = ("matchstar", "scanthru")


class NotFusable(ValueError):
    pass


# ----------------------------------------------------------------------------------------
# 1. while -> MatchStar
# ----------------------------------------------------------------------------------------

def _reads(stmts) -> Dict[str, int]:
    cnt: Dict[str, int] = {}
    for s in walk(stmts):
        if isinstance(s, Op):
            for a in s.args:
                cnt[a] = cnt.get(a, 0) + 1
        else:
            cnt[s.cond] = cnt.get(s.cond, 0) + 1
    return cnt


def _symbolic_body(body: Sequence, loop_vars: set):
    """Execute a straight-line loop body symbolically.  Values are nested tuples over the
    loop-entry values ('in', name) of variables assigned in the body and over invariant names."""
    env: Dict[str, tuple] = {}

    def val(name):
        if name in env:
            return env[name]
        if name in loop_vars:
            return ("in", name)
        return ("inv", name)

    for s in body:
        if not isinstance(s, Op):
            return None
        x = [val(a) for a in s.args]
        if s.op == "assign":
            env[s.dst] = x[0]
        elif s.op in ("and", "or", "xor"):
            env[s.dst] = (s.op, frozenset(x)) if x[0] != x[1] else x[0]
        elif s.op == "not":
            env[s.dst] = ("not", x[0])
        elif s.op == "advance":
            env[s.dst] = ("advance", x[0], s.shift)
        else:
            env[s.dst] = (s.op,) + tuple(x)
    return env


def _match_star_loop(w: While, prev: Sequence) -> Optional[Tuple[str, str, str, str]]:
    """If ``w`` is icgrep's unbounded character-class repetition loop, return
    (test, accum, start, cls)."""
    body = w.body
    if any(not isinstance(s, Op) for s in body):
        return None
    assigned = {s.dst for s in body}
    env = _symbolic_body(body, assigned)
    if env is None:
        return None
    test = w.cond
    if test not in env:
        return None
    for accum in assigned:
        if accum == test or accum not in env:
            continue
        for cls in _candidates(env[test]):
            step = ("advance", ("and", frozenset([("in", test), ("inv", cls)])), 1)
            want_test = ("and", frozenset([step, ("not", ("in", accum))]))
            want_acc = ("or", frozenset([step, ("in", accum)]))
            if env[test] == want_test and env[accum] == want_acc:
                start = _entry_value(prev, test, accum)
                if start is not None:
                    return test, accum, start, cls
    return None


def _candidates(expr):
    """Invariant names appearing in expr (candidate character classes)."""
    out = []

    def rec(e):
        if isinstance(e, tuple):
            if e and e[0] == "inv":
                out.append(e[1])
                return
            for x in e[1:]:
                if isinstance(x, frozenset):
                    for y in x:
                        rec(y)
                else:
                    rec(x)

    rec(expr)
    return out


def _entry_value(prev: Sequence, test: str, accum: str) -> Optional[str]:
    """Both loop variables must be copies of the same value when the loop is entered."""
    src = {}
    for s in reversed(prev):
        if isinstance(s, Op) and s.dst in (test, accum) and s.dst not in src:
            if s.op != "assign":
                return None
            src[s.dst] = s.args[0]
        elif not isinstance(s, Op):
            # a loop/if between the definition and this loop could redefine them
            if any(isinstance(x, Op) and x.dst in (test, accum) for x in walk([s])):
                return None
        if len(src) == 2:
            break
    if len(src) != 2 or src[test] != src[accum]:
        return None
    start = src[test]
    # start must not be redefined between its copy and the loop
    return start


def convert_star_loops(stmts: List, program_reads: Optional[Dict[str, int]] = None) -> List:
    """Replace recognised star loops by MatchStar, recursively; other statements unchanged."""
    if program_reads is None:
        program_reads = _reads(stmts)
    out: List = []
    for s in stmts:
        if isinstance(s, While):
            m = _match_star_loop(s, out)
            if m is not None:
                test, accum, start, cls = m
                temps = {x.dst for x in s.body} - {test, accum}
                inner = _reads(s.body)
                leaked = any(program_reads.get(t, 0) > inner.get(t, 0) for t in temps)
                if not leaked:
                    out.append(Op(accum, "matchstar", (start, cls)))
                    out.append(Op(test, "assign", ("0",)))
                    continue
            out.append(While(s.cond, convert_star_loops(s.body, program_reads)))
        elif isinstance(s, If):
            out.append(If(s.cond, convert_star_loops(s.then, program_reads),
                          convert_star_loops(s.orelse, program_reads) if s.orelse is not None else None))
        else:
            out.append(s)
    return out


def fusable(group: Group) -> bool:
    return all(isinstance(s, Op) for s in convert_star_loops(group.stmts))


# ----------------------------------------------------------------------------------------
# 2. SSA DAG
# ----------------------------------------------------------------------------------------

@dataclass
class Node:
    id: int
    op: str            # basis | zero | ones | and | or | xor | not | sel | advance | matchstar | scanthru
    args: Tuple[int, ...] = ()
    shift: int = 0
    basis: int = -1


class Dag:
    def __init__(self):
        self.nodes: List[Node] = []
        self.memo: Dict[tuple, int] = {}
        self.basis = [self._new(Node(0, "basis", basis=i)) for i in range(8)]
        self.zero = self._new(Node(0, "zero"))
        self.ones = self._new(Node(0, "ones"))

    def _new(self, n: Node) -> int:
        n.id = len(self.nodes)
        self.nodes.append(n)
        return n.id

    def make(self, op: str, args: Tuple[int, ...], shift: int = 0) -> int:
        z, o = self.zero, self.ones
        # constant folding keeps the skip analysis simple
        if op == "not":
            a = args[0]
            if a == z:
                return o
            if a == o:
                return z
            na = self.nodes[a]
            if na.op == "not":
                return na.args[0]
        elif op == "and":
            a, b = args
            if z in args:
                return z
            if a == o:
                return b
            if b == o or a == b:
                return a
            args = tuple(sorted(args))
        elif op == "or":
            a, b = args
            if o in args:
                return o
            if a == z:
                return b
            if b == z or a == b:
                return a
            args = tuple(sorted(args))
        elif op == "xor":
            a, b = args
            if a == b:
                return z
            if a == z:
                return b
            if b == z:
                return a
            args = tuple(sorted(args))
        elif op == "sel":
            c, a, b = args
            if a == b:
                return a
            if c == o:
                return a
            if c == z:
                return b
        elif op == "advance":
            if shift == 0 or args[0] == z:
                return args[0]
        elif op == "matchstar":
            m, c = args
            if m == z:
                return z
        elif op == "scanthru":
            m, c = args
            if m == z:
                return z
        key = (op, args, shift)
        hit = self.memo.get(key)
        if hit is not None:
            return hit
        nid = self._new(Node(0, op, args, shift))
        self.memo[key] = nid
        return nid

    def add_group(self, group: Group, names: Sequence[str]) -> List[int]:
        stmts = convert_star_loops(group.stmts)
        if not all(isinstance(s, Op) for s in stmts):
            raise NotFusable("program keeps while/if blocks that are not MatchStar loops")
        env: Dict[str, int] = {f"basis{i}": self.basis[i] for i in range(8)}
        env["0"] = self.zero
        env["1"] = self.ones
        for s in stmts:
            a = tuple(env[x] for x in s.args)
            if s.op == "assign":
                env[s.dst] = a[0]
            else:
                env[s.dst] = self.make(s.op, a, s.shift)
        return [env[n] for n in names]

    def is_cc(self, nid: int) -> bool:
        """True for pure character-class nodes (bitwise functions of the basis only)."""
        return self._cc[nid]

    def analyse(self):
        self._cc = []
        for n in self.nodes:
            if n.op in ("basis", "zero", "ones"):
                self._cc.append(True)
            elif n.op in ("and", "or", "xor", "not", "sel"):
                self._cc.append(all(self._cc[a] for a in n.args))
            else:
                self._cc.append(False)


# ----------------------------------------------------------------------------------------
# 3/4. Kernel generation
# ----------------------------------------------------------------------------------------

@dataclass
class Tuning:
    wpt: int = 2            # 32-bit words per lane
    block: int = 256        # threads per CTA
    skip_interval: int = 1  # check for an all-zero marker every k AND steps (0 = never)

    def key(self):
        return (self.wpt, self.block, self.skip_interval)


@dataclass
class KernelSpec:
    source: str
    name: str
    n_outputs: int
    n_adds: int
    halo_lanes: int
    wpt: int
    block: int
    max_depth_bits: int
    n_nodes: int
    output_names: List[str] = field(default_factory=list)

    @property
    def tile_words(self):
        return (32 - self.halo_lanes) * self.wpt

    def digest(self) -> str:
        return hashlib.sha256(self.source.encode()).hexdigest()[:16]


class _Gen:
    def __init__(self, dag: Dag, tuning: Tuning):
        self.d = dag
        self.t = tuning
        self.lines: List[str] = []
        self.indent = 2
        self.scopes: List[Dict[int, str]] = [{}]
        self.adds: Dict[int, int] = {}
        self.uses: Dict[int, int] = {}
        self.tmp = 0

    # analysis ---------------------------------------------------------------------------
    def analyse(self, outputs: Sequence[int]):
        d = self.d
        d.analyse()
        lane_bits = 32 * self.t.wpt
        self.dbits: Dict[int, int] = {}
        self.dl: Dict[int, int] = {}
        for n in d.nodes:
            if n.op in ("basis", "zero", "ones"):
                self.dbits[n.id] = 0
            elif n.op == "advance":
                self.dbits[n.id] = self.dbits[n.args[0]] + n.shift
            elif n.op in ADD_OPS:
                inb = max(self.dbits[a] for a in n.args)
                dl = -(-inb // lane_bits)
                self.dl[n.id] = dl
                self.dbits[n.id] = (dl + 1) * lane_bits
            else:
                self.dbits[n.id] = max(self.dbits[a] for a in n.args)
        live = set()
        stack = list(outputs)
        while stack:
            v = stack.pop()
            if v in live:
                continue
            live.add(v)
            stack.extend(d.nodes[v].args)
        self.live = live
        hl = 0
        for o in outputs:
            hl = max(hl, -(-self.dbits[o] // lane_bits))
        for v in live:
            if v in self.dl:
                hl = max(hl, self.dl[v] + 1)
        if hl >= 32:
            raise NotFusable(f"program depth needs {hl} halo lanes at {self.t.wpt} words/lane")
        self.hl = hl
        self.max_dbits = max([self.dbits[o] for o in outputs] + [0])
        for v in live:
            for a in d.nodes[v].args:
                self.uses[a] = self.uses.get(a, 0) + 1
        for o in outputs:
            self.uses[o] = self.uses.get(o, 0) + 1
        k = 0
        for v in sorted(live):
            if d.nodes[v].op in ADD_OPS:
                self.adds[v] = k
                k += 1

    # emission helpers -------------------------------------------------------------------
    def emit(self, s: str):
        self.lines.append(" " * self.indent + s)

    def lookup(self, v: int) -> Optional[str]:
        for sc in reversed(self.scopes):
            if v in sc:
                return sc[v]
        return None

    def open(self, cond: str):
        self.emit(f"if ({cond}) {{")
        self.indent += 2
        self.scopes.append({})

    def close(self):
        self.scopes.pop()
        self.indent -= 2
        self.emit("}")

    # scalar emission: a value is a name; word j of it is `{name}_{j}` (or a literal) -------
    def w(self, ref: str, j: int) -> str:
        if ref in ("0u", "0xffffffffu"):
            return ref
        return f"{ref}_{j}"

    def word_back(self, ref: str, J: int) -> str:
        """Word (lane*WPT + J) of `ref` as seen from this lane (J < 0 reads earlier lanes);
        words before the input start read as zero."""
        wpt = self.t.wpt
        if ref in ("0u",):
            return "0u"
        if J >= 0:
            return f"({self.w(ref, J)} & t.vm.w[{J}])"
        L = (-J + wpt - 1) // wpt
        I = J + L * wpt
        return f"__shfl_up_sync(FULL, {self.w(ref, I)} & t.vm.w[{I}], {L})"

    def emit_op(self, name: str, n: Node, a: List[str], declare: bool = True):
        wpt = self.t.wpt
        op = n.op
        pre = "const uint32_t " if declare else ""
        for j in range(wpt):
            x = [self.w(r, j) for r in a]
            if op == "and":
                e = f"{x[0]} & {x[1]}"
            elif op == "or":
                e = f"{x[0]} | {x[1]}"
            elif op == "xor":
                e = f"{x[0]} ^ {x[1]}"
            elif op == "not":
                e = f"~{x[0]}"
            elif op == "sel":
                e = f"({x[0]} & {x[1]}) | (~{x[0]} & {x[2]})"
            elif op == "advance":
                q, r = divmod(n.shift, 32)
                cur = self.word_back(a[0], j - q)
                if r == 0:
                    e = cur
                else:
                    prev = self.word_back(a[0], j - q - 1)
                    e = f"__funnelshift_r({cur}, {prev}, {r})"
            else:
                raise AssertionError(op)
            self.emit(f"{pre}{name}_{j} = {e};")

    def declare_zero(self, name: str):
        self.emit("uint32_t " + ", ".join(f"{name}_{j} = 0u" for j in range(self.t.wpt)) + ";")

    def any_expr(self, ref: str) -> str:
        ws = " | ".join(self.w(ref, j) for j in range(self.t.wpt))
        return f"__any_sync(FULL, ({ws}) != 0u)"

    def pack(self, ref: str) -> str:
        return "S{{" + ", ".join(self.w(ref, j) for j in range(self.t.wpt)) + "}}"

    # materialisation --------------------------------------------------------------------
    def mat(self, v: int) -> str:
        hit = self.lookup(v)
        if hit is not None:
            return hit
        n = self.d.nodes[v]
        if n.op == "basis":
            return f"b{n.basis}"
        if n.op == "zero":
            return "0u"
        if n.op == "ones":
            return "0xffffffffu"
        name = f"v{v}"
        if self.d.is_cc(v):
            a = [self.mat(x) for x in n.args]
            self.emit_op(name, n, a)
            self.scopes[-1][v] = name
            return name
        if n.op in ADD_OPS:
            m = self.mat(n.args[0])
            c = self.mat(n.args[1])
            fn = "matchstar" if n.op == "matchstar" else "scanthru"
            self.emit(f"const S {name}_s = {fn}<{self.dl[v]}>(p, t, {self.adds[v]}, {self.pack(m)}, {self.pack(c)});")
            for j in range(self.t.wpt):
                self.emit(f"const uint32_t {name}_{j} = {name}_s.w[{j}];")
            self.scopes[-1][v] = name
            return name
        if n.op in CHAIN_OPS:
            return self.mat_chain(v)
        a = [self.mat(x) for x in n.args]
        self.emit_op(name, n, a)
        self.scopes[-1][v] = name
        return name

    def chain_operand(self, v: int) -> Optional[int]:
        n = self.d.nodes[v]
        if n.op == "advance":
            return n.args[0]
        if n.op == "and":
            a, b = n.args
            ca, cb = self.d.is_cc(a), self.d.is_cc(b)
            if ca and not cb:
                return b
            if cb and not ca:
                return a
            if not ca and not cb:
                return a if self.dbits[a] >= self.dbits[b] else b
        return None

    def mat_chain(self, v: int) -> str:
        d = self.d
        chain = [v]
        u = self.chain_operand(v)
        while (u is not None and d.nodes[u].op in CHAIN_OPS and not d.is_cc(u)
               and self.uses.get(u, 0) <= 1 and self.lookup(u) is None):
            chain.append(u)
            u = self.chain_operand(u)
        root = u
        rname = self.mat(root)
        # heavy side operands must exist before the guarded blocks open
        side: Dict[int, int] = {}
        for c in chain:
            n = d.nodes[c]
            if n.op == "and":
                other = n.args[1] if self.chain_operand(c) == n.args[0] else n.args[0]
                side[c] = other
                if not d.is_cc(other):
                    self.mat(other)
        name = f"v{v}"
        self.declare_zero(name)
        depth = 0
        prev = rname
        ands = 0
        k = self.t.skip_interval
        for c in reversed(chain):
            n = d.nodes[c]
            if n.op == "and":
                if k > 0 and ands % k == 0:
                    self.open(self.any_expr(prev))
                    depth += 1
                ands += 1
                a = [prev, self.mat(side[c])]
            else:
                a = [prev]
            if c == v:
                self.emit_op(name, n, a, declare=False)
            else:
                tmp = f"v{c}"
                self.emit_op(tmp, n, a)
                prev = tmp
        for _ in range(depth):
            self.close()
        self.scopes[-1][v] = name
        return name

    # kernel pieces ---------------------------------------------------------------------------
    def body(self, outputs: Sequence[int], out_names: Sequence[str], out_base: int) -> str:
        """Code computing and storing `outputs` (analyse() must have run)."""
        self.lines = []
        self.indent = 2
        self.scopes = [{}]
        for i, (o, nm) in enumerate(zip(outputs, out_names)):
            self.emit(f"/* output {out_base + i}: {nm} */")
            r = self.mat(o)
            self.emit(f"store(p, t, {out_base + i}, {self.pack(r)});")
        return "\n".join(self.lines)


def _basis_params(wpt: int) -> str:
    return ", ".join(f"uint32_t b{i}_{j}" for i in range(8) for j in range(wpt))


def _basis_args(wpt: int) -> str:
    return ", ".join(f"b[{i}].w[{j}]" for i in range(8) for j in range(wpt))


def build_dag(groups: Sequence[Group], per_regex: bool = False) -> Tuple[Dag, List[int], List[str]]:
    dag = Dag()
    outs: List[int] = []
    names: List[str] = []
    for gi, g in enumerate(groups):
        if per_regex and g.regex_results:
            ids = dag.add_group(g, g.regex_results)
            outs.extend(ids)
            labels = g.regexes or g.regex_results
            names.extend(f"group {gi} regex {j}: {labels[j]}" for j in range(len(ids)))
        else:
            outs.extend(dag.add_group(g, [g.result]))
            names.append(f"group {gi}")
    return dag, outs, names


def generate_kernel(groups: Sequence[Group], tuning: Optional[Tuning] = None,
                    per_regex: bool = False, name: str = "bg_scan") -> KernelSpec:
    """Lower the pattern set into one kernel: one non-inlined device function per group (so
    compile time grows linearly and NVRTC can split the work across threads), called in turn on
    every tile after the tile's bytes are loaded and transposed once."""
    tuning = tuning or Tuning()
    parts = []
    hl = 0
    max_dbits = 0
    n_nodes = 0
    names_all: List[str] = []
    for gi, g in enumerate(groups):
        dag, outs, names = build_dag([g], per_regex)
        names = [nm.replace("group 0", f"group {gi}", 1) for nm in names]
        gen = _Gen(dag, tuning)
        gen.analyse(outs)
        hl = max(hl, gen.hl)
        max_dbits = max(max_dbits, gen.max_dbits)
        n_nodes += len(dag.nodes)
        parts.append((gen, outs, names))
    add_base = 0
    out_base = 0
    funcs = []
    wpt = tuning.wpt
    for gi, (gen, outs, names) in enumerate(parts):
        gen.adds = {v: add_base + k for v, k in gen.adds.items()}
        add_base += len(gen.adds)
        code = gen.body(outs, [nm.replace("*/", "* /") for nm in names], out_base)
        out_base += len(outs)
        names_all.extend(names)
        funcs.append(
            f"__device__ __noinline__ void bg_group_{gi}(const BgParams &p, const Tile &t, {_basis_params(wpt)}) {{\n"
            f"{code}\n}}\n")
    calls = "\n".join(f"    bg_group_{gi}(p, t, {_basis_args(wpt)});" for gi in range(len(parts)))
    src = (
        f"#define BG_WPT {wpt}\n"
        f"#define BG_HL {hl}\n"
        f'#include "bg_device.cuh"\n'
        f"using namespace bg;\n"
        + "\n".join(funcs) +
        f'extern "C" __global__ void __launch_bounds__({tuning.block}) {name}(const __grid_constant__ BgParams p) {{\n'
        f"  Tile t;\n"
        f"  init(p, t);\n"
        f"  while (next_tile(p, t)) {{\n"
        f"    S b[8];\n"
        f"    load_basis(p, t, b);\n"
        f"{calls}\n"
        f"  }}\n"
        f"}}\n"
    )
    return KernelSpec(source=src, name=name, n_outputs=out_base, n_adds=add_base,
                      halo_lanes=hl, wpt=wpt, block=tuning.block, max_depth_bits=max_dbits,
                      n_nodes=n_nodes, output_names=names_all)
