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
import sys
from dataclasses import dataclass, field, replace
from typing import Dict, List, Optional, Sequence, Tuple

from . import prefilter
from .pablo import BASIS, Group, If, Op, While, walk

CHAIN_OPS = ("and", "advance")
ADD_OPS = ("matchstar", "scanthru")


class _OrderError(Exception):
    """A part's zero-skip regions would read a node before the code computing it has run."""


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


def push_advances(dag: Dag, outs: Sequence[int]) -> List[int]:
    """Rewrite the outputs so that Advances sit on character classes.

    A shift distributes over AND, OR and XOR exactly (zeros shift in at the input start either
    way), and consecutive shifts add up, so ``Advance(Advance(m, 1) & C, 1) & D`` becomes
    ``Advance(m, 2) & Advance(C, 1) & D``.  A concatenation of classes then costs one AND per
    position on class streams shifted once per (class, distance), shared by every pattern
    that reads the class at that distance, instead of a shift of the running marker per
    position.  The rewrite goes through a node only where it has one user (or at distance 0),
    so no work is duplicated: a shared node is computed once and its result shifted, as
    before.  Other operations (NOT, SEL, the additions, look-aheads) are rebuilt over their
    rewritten operands."""
    dag.analyse()
    cc = list(dag._cc)
    uses: Dict[int, int] = {}
    live, stack = set(), list(outs)
    while stack:
        v = stack.pop()
        if v in live:
            continue
        live.add(v)
        stack.extend(dag.nodes[v].args)
    for v in live:
        for a in dag.nodes[v].args:
            uses[a] = uses.get(a, 0) + 1
    for o in outs:
        uses[o] = uses.get(o, 0) + 1
    memo: Dict[Tuple[int, int], int] = {}

    def push(v: int, s: int) -> int:
        key = (v, s)
        hit = memo.get(key)
        if hit is not None:
            return hit
        n = dag.nodes[v]
        through = s == 0 or uses.get(v, 0) <= 1
        if cc[v]:
            r = dag.make("advance", (v,), s)
        elif n.op == "advance" and through:
            r = push(n.args[0], s + n.shift)
        elif n.op in ("and", "or", "xor") and through:
            r = dag.make(n.op, (push(n.args[0], s), push(n.args[1], s)))
        elif s == 0:
            r = dag.make(n.op, tuple(push(a, 0) for a in n.args), n.shift)
        else:
            u = push(v, 0)
            if dag.nodes[u].op == "advance":    # shifts add up
                r = dag.make("advance", dag.nodes[u].args, dag.nodes[u].shift + s)
            else:
                r = dag.make("advance", (u,), s)
        memo[key] = r
        return r

    limit = sys.getrecursionlimit()
    sys.setrecursionlimit(max(limit, 20 * len(dag.nodes) + 1000))
    try:
        out = [push(o, 0) for o in outs]
    finally:
        sys.setrecursionlimit(limit)
    dag.analyse()
    return out


def _cluster_chains(members: List[int], leaves: Dict[int, List[Tuple[int, int]]],
                    batch: int) -> List[List[int]]:
    """Split chains into batches of at most `batch` that share shifted classes: each batch
    starts from the remaining chain with the most leaves and greedily takes the chain whose
    leaves are most often already in the batch (ties: fewer new leaves, then lower id), so
    that a batch computes fewer distinct shifted classes.  Beyond 512 chains the chains keep
    their order (the greedy search is quadratic)."""
    if len(members) <= batch or len(members) > 512:
        return [members[i:i + batch] for i in range(0, len(members), batch)]
    sets = {r: set(leaves[r]) for r in members}
    left = sorted(members)
    out = []
    while left:
        seed = max(left, key=lambda r: (len(sets[r]), -r))
        grp, have = [seed], set(sets[seed])
        left.remove(seed)
        while left and len(grp) < batch:
            best = max(left, key=lambda r: (len(sets[r] & have), -len(sets[r] - have), -r))
            grp.append(best)
            have |= sets[best]
            left.remove(best)
        out.append(sorted(grp))
    return out


def _shared_pairs(leaf_sets: Dict[int, List[Tuple[int, int]]]) -> Dict[int, List[Tuple]]:
    """Per chain of a batch, the pairs of its shifted classes that it ANDs through a node shared
    with other chains of the batch: greedily the pair most chains hold, while two or more do,
    each class of a chain in one pair at most."""
    free = {r: set(ls) for r, ls in leaf_sets.items()}
    out: Dict[int, List[Tuple]] = {r: [] for r in leaf_sets}
    while True:
        count: Dict[Tuple, int] = {}
        for r, ls in free.items():
            srt = sorted(ls)
            for i in range(len(srt)):
                for j in range(i + 1, len(srt)):
                    count[(srt[i], srt[j])] = count.get((srt[i], srt[j]), 0) + 1
        best = max(count.items(), key=lambda kv: (kv[1], kv[0]), default=None)
        if best is None or best[1] < 2:
            return out
        pair = best[0]
        for r, ls in free.items():
            if pair[0] in ls and pair[1] in ls:
                ls.discard(pair[0])
                ls.discard(pair[1])
                out[r].append(pair)


def interleave_chains(dag: Dag, outs: Sequence[int], batch: int,
                      pairs: bool = False) -> Tuple[List[int], Dict[int, int]]:
    """Re-associate the AND chains of a pushed program distance-major.

    After ``push_advances`` a pattern is an AND of shifted classes ``Advance(C, d)`` (and of
    a few shared markers).  Computed pattern by pattern, a shifted class that several patterns
    read must either be recomputed or held in a register from its first to its last use.  Here
    the chains (maximal trees of single-use ANDs) are rebuilt together, `batch` chains at a
    time: for each distance d, largest first, every class shifted by d is computed once and
    ANDed into each chain of the batch that reads it; the chain's other operands (shared
    markers, ORs, additions) are ANDed in last.  A chain that reads another chain's result is
    built in a later wave than that chain.  AND is associative and commutative, so the values
    are unchanged.  Returns the new outputs and, for each AND node built here, its batch
    number (the code generator shares a shifted class within a batch).  With `pairs`, two
    shifted classes that several chains of a batch read are ANDed once into a node those chains
    share (`_shared_pairs`), at the distance of the later of the two."""
    dag.analyse()
    cc = dag._cc
    live, stack = set(), list(outs)
    while stack:
        v = stack.pop()
        if v in live:
            continue
        live.add(v)
        stack.extend(dag.nodes[v].args)
    users: Dict[int, List[int]] = {}
    for v in live:
        for a in dag.nodes[v].args:
            users.setdefault(a, []).append(v)

    def is_and(v):
        return dag.nodes[v].op == "and" and not cc[v]

    def leaf(v):
        """(class, distance) of a shifted class, else None."""
        n = dag.nodes[v]
        if cc[v]:
            return (v, 0)
        if n.op == "advance" and cc[n.args[0]]:
            return (n.args[0], n.shift)
        return None

    out_set = set(outs)

    def inner(v):   # an AND folded into its single user's chain
        return (is_and(v) and v not in out_set and len(users.get(v, ())) == 1
                and is_and(users[v][0]))

    roots = [v for v in sorted(live) if is_and(v) and not inner(v)]
    flat: Dict[int, Tuple[List[Tuple[int, int]], List[int]]] = {}
    for r in roots:
        leaves, others, st = [], [], list(dag.nodes[r].args)
        while st:
            a = st.pop()
            if inner(a):
                st.extend(dag.nodes[a].args)
            elif leaf(a) is not None:
                leaves.append(leaf(a))
            else:
                others.append(a)
        flat[r] = (leaves, others)
    root_set = set(roots)
    need_memo: Dict[int, int] = {}
    wave: Dict[int, int] = {}

    def need(x):
        if x in need_memo:
            return need_memo[x]
        if leaf(x) is not None:
            r = 0
        elif x in root_set:
            r = wave_of(x) + 1
        else:
            r = max([need(a) for a in dag.nodes[x].args] + [0])
        need_memo[x] = r
        return r

    def wave_of(r):
        if r not in wave:
            wave[r] = max([need(o) for o in flat[r][1]] + [0])
        return wave[r]

    built: Dict[int, int] = {}
    memo: Dict[int, int] = {}

    def rebuild(v):
        if v in built:
            return built[v]
        if leaf(v) is not None:
            return v
        if v in memo:
            return memo[v]
        n = dag.nodes[v]
        assert v not in root_set, "chain used before its wave"
        r = dag.make(n.op, tuple(rebuild(a) for a in n.args), n.shift)
        memo[v] = r
        return r

    def fresh_and(a, b):
        """A new AND node (no hash-consing: the pushed chains' own nodes hold the same
        operands, and the code generator emits nodes in creation order)."""
        if dag.zero in (a, b):
            return dag.zero
        if a == dag.ones:
            return b
        if b == dag.ones:
            return a
        return dag._new(Node(0, "and", (a, b)))

    epochs: Dict[int, int] = {}
    limit = sys.getrecursionlimit()
    sys.setrecursionlimit(max(limit, 20 * len(dag.nodes) + 1000))
    try:
        for r in roots:
            wave_of(r)
        k = 0
        steps = [g for w in sorted(set(wave.values()))
                 for g in _cluster_chains([r for r in roots if wave[r] == w],
                                          {r: flat[r][0] for r in roots}, max(1, batch))]
        for grp in steps:
            acc: Dict[int, Optional[int]] = {r: None for r in grp}
            dists = sorted({d for r in grp for _, d in flat[r][0]}, reverse=True)
            by_d = {r: {} for r in grp}
            for r in grp:
                for c, d in flat[r][0]:
                    by_d[r].setdefault(d, []).append(c)
            # shared pairs: a chain ANDs a pair's node in place of its two classes, at the pair's
            # later distance (the smaller d; ties: the larger class)
            paired: Dict[int, Dict[Tuple[int, int], Optional[Tuple]]] = {r: {} for r in grp}
            if pairs:
                for r, prs in _shared_pairs({r: flat[r][0] for r in grp}).items():
                    for a_, b_ in prs:
                        late = min(a_, b_, key=lambda x: (x[1], -x[0]))
                        paired[r][a_] = (a_, b_) if a_ == late else None
                        paired[r][b_] = (a_, b_) if b_ == late else None
            pair_node: Dict[Tuple, int] = {}

            def operand_at(r, c, d):
                lf = (c, d)
                if lf not in paired[r]:
                    return dag.make("advance", (c,), d)
                pr = paired[r][lf]
                if pr is None:          # the pair is ANDed at its other class's distance
                    return None
                if pr not in pair_node:
                    pa, pb = (dag.make("advance", (x[0],), x[1]) for x in pr)
                    pair_node[pr] = fresh_and(pa, pb)
                    epochs.setdefault(pair_node[pr], k)
                return pair_node[pr]

            for d in dists:
                for r in grp:
                    for c in sorted(by_d[r].get(d, [])):
                        lf = operand_at(r, c, d)
                        if lf is None:
                            continue
                        if acc[r] is None:
                            acc[r] = lf
                        else:
                            acc[r] = fresh_and(acc[r], lf)
                            epochs.setdefault(acc[r], k)
            for r in grp:
                for o in flat[r][1]:
                    ro = rebuild(o)
                    if acc[r] is None:
                        acc[r] = ro
                    else:
                        acc[r] = fresh_and(acc[r], ro)
                        epochs.setdefault(acc[r], k)
                built[r] = acc[r]
            k += 1
        new = [rebuild(o) for o in outs]
    finally:
        sys.setrecursionlimit(limit)
    dag.analyse()
    return new, epochs


# ----------------------------------------------------------------------------------------
# 3/4. Kernel generation
# ----------------------------------------------------------------------------------------

@dataclass
class Tuning:
    wpt: int = 1            # 32-bit words per lane
    block: int = 256        # threads per CTA
    skip_interval: int = -1  # check for an all-zero marker every k AND steps (0 = never; -1:
                             # never in the split form, whose tiles mostly hold the marker's
                             # q-gram, nor when unselective filters choose the single-kernel
                             # form; every AND when the single-kernel form is forced)
    part_cap: int = 0       # most OR-ed terms one part function computes (0: 2 in the split
                            # form, 64 in the single-kernel form)
    window: int = 2         # guard blocks kept pending (instruction-level parallelism vs registers)
    min_blocks: int = 3     # __launch_bounds__ minimum resident blocks per SM (caps registers)
    edge_variants: bool = False  # separate unmasked part code for tiles away from input ends
    inline_lookback: bool = False  # look-back code inlined at each addition (else one shared function)
    lockstep: bool = False  # warps of a block run each part together (barrier between parts)
    lookback_width: int = 1  # predecessor records each lane examines per look-back step
    lookback_spin: int = 0   # look-back polls before sleeping
    carry_prepass: bool = True  # carries of wide-class additions from a pre-pass, not look-back
    prefilter: bool = True   # run a term only in tiles holding one of its q-grams
    bloom_bits: int = 20     # prefilter: log2 of the Bloom bitmap's size (shared memory)
    cls_block: int = 1024    # split form: threads per classify block (one block per SM holds
                             # the Bloom bitmap, the exact keys and the warps' run masks)
    prefilter_limit: float = 0.25  # prefilter only while a tile is expected to run fewer than
                                   # this fraction of the terms and to take fewer than 8 times
                                   # this many Bloom hits per 1024 bytes (text taken as uniform
                                   # over the bytes the filters name); >= 1: always
    merge_outputs: bool = True   # split form: parts of part_cap terms, outputs merged by atomicOr
    exec_groups: int = 16    # split form: SM groups of the execute pass (each starts on its own parts)
    exec_claim: int = 1      # split form: work items an execute warp claims at once
    exec_min_blocks: int = 4     # split form: min_blocks of the execute kernel (its loads wait on
                                 # HBM, so more warps beat more registers; 0: min_blocks)
    inline_parts: int = 160  # split form: inline the parts into the execute kernel up to this many
    single_wpt: int = 1      # words per lane (and blocks per SM below) when the compiler falls
    single_min_blocks: int = 2   # back to the single-kernel form because the filters are
                                 # unselective (0: keep wpt / min_blocks); 2 blocks of 256
                                 # give the distance-major chains 128 registers a thread
    single_edge: bool = True     # that form also gets unmasked part code for tiles that touch
                                 # no input end (edge_variants)
    basis_filter: bool = True    # split form: rebuild the bytes of basis-plane inputs and run
                                 # the q-gram filter on them (else every term runs there)
    filter_config: Optional[Tuple[int, int]] = None  # prefilter (q-gram length, stride); None:
                                                     # the cheapest by the filter's cost model
    bulk_zero: bool = True   # split form: classify zeroes the outputs with bulk copies from
                             # shared memory (else with vector stores of its lanes)
    push_advances: bool = True   # single-kernel form: Advances pushed through single-use
                                 # AND/OR/XOR down to the character classes, each class shifted
                                 # once per distance; a word read from another lane is shared
    claim_tiles: int = 4         # single-kernel form: consecutive tiles a warp claims at once
    chain_batch: int = 8         # with push_advances: AND chains re-associated distance-major,
                                 # this many at a time (0: each chain computed on its own)
    pair_share: bool = True      # with chain_batch: pairs of shifted classes that several chains
                                 # of a batch read are ANDed once (interleave_chains(pairs=));
                                 # 64 DNA motifs: 2% faster

    def key(self):
        return (self.wpt, self.block, self.skip_interval, self.part_cap, self.window,
                self.min_blocks, self.edge_variants, self.inline_lookback, self.lockstep,
                self.lookback_width, self.lookback_spin, self.carry_prepass, self.prefilter,
                self.merge_outputs, self.bloom_bits, self.prefilter_limit, self.exec_groups,
                self.cls_block, self.single_wpt, self.single_min_blocks, self.inline_parts,
                self.basis_filter, self.filter_config, self.bulk_zero, self.exec_claim,
                self.exec_min_blocks,
                self.push_advances, self.chain_batch, self.single_edge, self.claim_tiles,
                self.pair_share)


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
    tail_lanes: int = 0
    n_pre: int = 0          # additions 0..n_pre-1 take their carries from the pre-pass kernel
    n_run: int = 0          # split form: run-mask words per tile (0 = single-kernel form)
    merges: bool = False    # parts OR into shared outputs: launches need the output streams
    n_parts: int = 0        # split form: part functions
    part_outputs: List[List[int]] = field(default_factory=list)  # split form: outputs of each part

    @property
    def tile_words(self):
        return (32 - self.halo_lanes - self.tail_lanes) * self.wpt

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
        self.pre: Dict[int, int] = {}   # pre-pass additions -> their index (= add index)
        self.uses: Dict[int, int] = {}
        self.tmp = 0
        self.share_reads = False
        self.inline: Dict[str, List[str]] = {}   # pseudo-values: per-word expressions
        self.epochs: Dict[int, int] = {}   # AND node -> batch of chains (interleave_chains)
        self.epoch = -1                    # batch of the node being computed
        self._order = None                 # (a part's heavy nodes, those computed so far)

    # analysis ---------------------------------------------------------------------------
    def byteset(self, v: int) -> int:
        """256-bit set of the byte values a character-class node is true for."""
        memo = self._bs
        if v in memo:
            return memo[v]
        n = self.d.nodes[v]
        full = (1 << 256) - 1
        if n.op == "basis":
            r = sum(1 << b for b in range(256) if (b >> (7 - n.basis)) & 1)
        elif n.op == "zero":
            r = 0
        elif n.op == "ones":
            r = full
        else:
            a = [self.byteset(x) for x in n.args]
            r = {"and": lambda: a[0] & a[1], "or": lambda: a[0] | a[1], "xor": lambda: a[0] ^ a[1],
                 "not": lambda: ~a[0] & full,
                 "sel": lambda: (a[0] & a[1]) | (~a[0] & a[2] & full)}[n.op]()
        memo[v] = r
        return r

    def wide_class(self, v: int) -> bool:
        """True if the class almost surely covers whole words of text (e.g. '.', '[^x]'), so
        an addition over it will usually need its predecessor's carry."""
        if not self.d.is_cc(v):
            return True
        bs = self.byteset(v)
        printable = sum(1 for b in range(0x20, 0x7F) if (bs >> b) & 1)
        return printable >= 90 or bin(bs).count("1") >= 200

    def analyse(self, outputs: Sequence[int]):
        d = self.d
        d.analyse()
        self._bs: Dict[int, int] = {}
        lane_bits = 32 * self.t.wpt
        self.dbits: Dict[int, int] = {}
        self.fbits: Dict[int, int] = {}
        self.dl: Dict[int, int] = {}
        for n in d.nodes:
            if n.op in ("basis", "zero", "ones"):
                self.fbits[n.id] = 0
            elif n.op == "lookahead":
                self.fbits[n.id] = self.fbits[n.args[0]] + n.shift
            else:
                self.fbits[n.id] = max(self.fbits[a] for a in n.args)
        for n in d.nodes:
            if n.op in ("basis", "zero", "ones"):
                self.dbits[n.id] = 0
            elif n.op == "lookahead":
                self.dbits[n.id] = self.dbits[n.args[0]]
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
        tl = 0
        for v in live:
            tl = max(tl, -(-self.fbits[v] // lane_bits))
        if hl + tl >= 32:
            raise NotFusable(f"program depth needs {hl} + {tl} halo lanes at {self.t.wpt} words/lane")
        self.hl = hl
        self.tl = tl
        self.max_dbits = max([self.dbits[o] for o in outputs] + [0])
        for v in live:
            for a in d.nodes[v].args:
                self.uses[a] = self.uses.get(a, 0) + 1
        for o in outputs:
            self.uses[o] = self.uses.get(o, 0) + 1
        # additions over a wide class whose operands depend on no other addition get their
        # carries from the pre-pass; they are numbered first
        pre = []
        if self.t.carry_prepass:
            for v in sorted(live):
                n = d.nodes[v]
                if n.op in ADD_OPS and self.wide_class(n.args[1]):
                    anc = self.heavy_ancestors(n.args[0]) | self.heavy_ancestors(n.args[1])
                    if not any(d.nodes[a].op in ADD_OPS for a in anc):
                        pre.append(v)
        k = 0
        for v in pre:
            self.adds[v] = k
            self.pre[v] = k
            k += 1
        for v in sorted(live):
            if d.nodes[v].op in ADD_OPS and v not in self.pre:
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
        e = self.inline.get(ref)
        if e is not None:
            return e[j]
        return f"{ref}_{j}"

    def operand(self, v: int) -> str:
        """Operand `v` of a bitwise operation on markers.  With shared reads on, a character
        class is read through its masked words (the reads its shifts use): the mask clears
        only positions before the input start, which no output keeps and every shift and
        addition clears again, so one copy of the class stays live instead of two."""
        n = self.d.nodes[v]
        if not (self.share_reads and self.d.is_cc(v) and n.op not in ("zero", "ones")):
            return self.mat(v)
        c = self.mat(v)
        name = f"@cls{self.tmp}"
        self.tmp += 1
        self.inline[name] = [self.shared(self.word_back(c, j)) for j in range(self.t.wpt)]
        return name

    def leaf(self, v: int) -> bool:
        """A shifted character class, recomputed at each use from the shared reads of its
        class (one funnel shift a word) instead of held in registers across the part."""
        n = self.d.nodes[v]
        return self.share_reads and n.op == "advance" and self.d.is_cc(n.args[0])

    def word_back(self, ref: str, J: int) -> str:
        """Word (lane*WPT + J) of `ref` as seen from this lane (J < 0 reads earlier lanes);
        words before the input start read as zero."""
        wpt = self.t.wpt
        if ref in ("0u",):
            return "0u"
        if J >= 0:
            return f"({self.w(ref, J)} & VM({J}))"
        L = (-J + wpt - 1) // wpt
        I = J + L * wpt
        return f"__shfl_up_sync(FULL, {self.w(ref, I)} & VM({I}), {L})"

    def word_fwd(self, ref: str, J: int) -> str:
        """Word (lane*WPT + J) of `ref` for J >= 0 (later lanes via shuffle down); positions at
        or beyond the end of the input read as zero."""
        wpt = self.t.wpt
        if ref in ("0u",):
            return "0u"
        if J < wpt:
            return f"({self.w(ref, J)} & EM({J}))"
        L, I = divmod(J, wpt)
        return f"__shfl_down_sync(FULL, {self.w(ref, I)} & EM({I}), {L})"

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
            elif op == "lookahead":
                q, r = divmod(n.shift, 32)
                cur = self.word_fwd(a[0], j + q)
                if r == 0:
                    e = cur
                else:
                    nxt = self.word_fwd(a[0], j + q + 1)
                    e = f"__funnelshift_l({nxt}, {cur}, {r})"
            elif op == "advance":
                q, r = divmod(n.shift, 32)
                cur = self.shared(self.word_back(a[0], j - q))
                if r == 0:
                    e = cur
                else:
                    prev = self.shared(self.word_back(a[0], j - q - 1))
                    e = f"__funnelshift_r({cur}, {prev}, {r})"
            else:
                raise AssertionError(op)
            self.emit(f"{pre}{name}_{j} = {e};")

    def shared(self, expr: str) -> str:
        """With shared reads on, a temporary holding `expr` (a masked word or a word read from
        another lane), declared once per scope, so that every shift of a class reuses it."""
        if not self.share_reads or expr in ("0u", "0xffffffffu"):
            return expr
        key = ("read", expr)
        for sc in reversed(self.scopes):
            if key in sc:
                return sc[key]
        name = f"sr{self.tmp}"
        self.tmp += 1
        self.emit(f"const uint32_t {name} = {expr};")
        self.scopes[-1][key] = name
        return name

    def declare_zero(self, name: str):
        self.emit("uint32_t " + ", ".join(f"{name}_{j} = 0u" for j in range(self.t.wpt)) + ";")

    def any_expr(self, ref: str) -> str:
        ws = " | ".join(self.w(ref, j) for j in range(self.t.wpt))
        return f"__any_sync(FULL, ({ws}) != 0u)"

    def pack(self, ref: str) -> str:
        return "S{{" + ", ".join(self.w(ref, j) for j in range(self.t.wpt)) + "}}"

    # materialisation --------------------------------------------------------------------
    def mat(self, v: int) -> str:
        order = self._order
        if order is not None and v in order[2] and v not in order[1]:
            # declared for a later guarded block and still its zero there: not readable yet
            # (anything else not computed yet is recomputed here from its operands)
            raise _OrderError(v)
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
        if self.leaf(v):
            key = ("leaf", v, self.epoch)
            if self.epoch >= 0:
                for sc in reversed(self.scopes):
                    if key in sc:
                        return sc[key]
            c = self.mat(n.args[0])
            q, r = divmod(n.shift, 32)
            exprs = []
            for j in range(self.t.wpt):
                cur = self.shared(self.word_back(c, j - q))
                if r == 0:
                    exprs.append(cur)
                else:
                    prev = self.shared(self.word_back(c, j - q - 1))
                    exprs.append(f"shr_funnel<{r}>({cur}, {prev})")
            if self.epoch >= 0:     # one temporary per batch, read by its chains
                name = f"lf{self.tmp}"
                self.tmp += 1
                for j, e in enumerate(exprs):
                    self.emit(f"const uint32_t {name}_{j} = {e};")
                self.scopes[-1][key] = name
                return name
            name = f"@leaf{self.tmp}"
            self.tmp += 1
            self.inline[name] = exprs
            return name
        name = f"v{v}"
        if self.d.is_cc(v):
            a = [self.mat(x) for x in n.args]
            self.emit_op(name, n, a)
            self.scopes[-1][v] = name
            return name
        if n.op in ADD_OPS:
            m = self.mat(n.args[0])
            c = self.mat(n.args[1])
            if v in self.pre:
                mode = 0 if n.op == "matchstar" else 1
                args = f"p, t, {self.adds[v]}, {mode}"
                self.emit(f"const AddState st{v} = add_known<{self.dl[v]}>({args}, {self.pack(m)}, {self.pack(c)});")
                self.emit(f"const S {name}_s = add_end<{self.dl[v]}>({args}, st{v}, {self.pack(m)}, {self.pack(c)});")
            else:
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

    def mat_chain(self, v: int, acc: Optional[List[str]] = None) -> Optional[str]:
        """Emit the chain of zero-preserving steps ending in `v` under zero-skip guards.  With
        `acc`, OR the value into those accumulators inside the innermost guard instead of
        returning it."""
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
        if acc is None:
            self.declare_zero(name)
        depth = 0
        prev = rname
        ands = 0
        k = self.t.skip_interval
        for c in reversed(chain):
            n = d.nodes[c]
            if n.op == "and":
                # the step before the first AND is dense (a class, one Advance); guards start
                # after the first AND and then repeat every k ANDs
                if k > 0 and ands >= 1 and (ands - 1) % k == 0:
                    self.open(self.any_expr(prev))
                    depth += 1
                ands += 1
                a = [prev, self.mat(side[c])]
            else:
                a = [prev]
            if c == v and acc is None:
                self.emit_op(name, n, a, declare=False)
            else:
                tmp = f"v{c}"
                self.emit_op(tmp, n, a)
                prev = tmp
        if acc is not None:
            for a_ in acc:
                for j in range(self.t.wpt):
                    self.emit(f"{a_}_{j} |= {name}_{j};")
        for _ in range(depth):
            self.close()
        if acc is not None:
            return None
        self.scopes[-1][v] = name
        return name

    def first_and(self, v: int) -> Optional[int]:
        """The first AND (closest to the root) of the single-use chain ending in `v`."""
        d = self.d
        u, found = v, None
        while (u is not None and d.nodes[u].op in CHAIN_OPS and not d.is_cc(u)
               and (u == v or self.uses.get(u, 0) <= 1) and self.lookup(u) is None):
            if d.nodes[u].op == "and":
                found = u
            u = self.chain_operand(u)
        return found

    def accumulate(self, v: int, accs: List[str]):
        """OR node `v` into accumulators; a single-use chain accumulates inside its guards."""
        n = self.d.nodes[v]
        if (self.lookup(v) is None and n.op in CHAIN_OPS and not self.d.is_cc(v)
                and self.uses.get(v, 0) <= 1):
            self.mat_chain(v, acc=accs)
            return
        r = self.mat(v)
        if r == "0u":
            return
        for a_ in accs:
            for j in range(self.t.wpt):
                self.emit(f"{a_}_{j} |= {self.w(r, j)};")

    def or_leaves(self, v: int) -> List[int]:
        """Split an output into the OR-ed terms it is made of (single-use OR nodes only)."""
        n = self.d.nodes[v]
        if n.op == "or" and not self.d.is_cc(v) and self.uses.get(v, 0) <= 1:
            return self.or_leaves(n.args[0]) + self.or_leaves(n.args[1])
        return [v]

    def heavy_ancestors(self, v: int) -> set:
        out, stack = set(), [v]
        while stack:
            x = stack.pop()
            if x in out or self.d.is_cc(x) or self.leaf(x):
                continue
            out.add(x)
            stack.extend(self.d.nodes[x].args)
        return out

    def pre_body(self) -> str:
        """Body of the pre-pass kernel: the operands of every pre-pass addition (with the same
        zero-skip guards as the main pass) and the publication of its tile aggregate."""
        self.lines = []
        self.indent = 4
        self.scopes = [{}]
        for v, k in sorted(self.pre.items(), key=lambda x: x[1]):
            n = self.d.nodes[v]
            m, c = self.mat(n.args[0]), self.mat(n.args[1])
            mode = 0 if n.op == "matchstar" else 1
            self.emit(f"{{ uint32_t G, P; pre_aggregate<{self.dl[v]}, E>(t, {mode}, {self.pack(m)}, {self.pack(c)}, G, P); "
                      f"pg[{k >> 5}] |= G << {k & 31}; pp[{k >> 5}] |= P << {k & 31}; }}")
        return "\n".join(self.lines)

    def part(self, terms: Sequence[Tuple[int, int]], outer_regs: bool = False) -> str:
        """`_part` with zero-block skipping, or, where its guard regions would order a read of
        a node before its computation (a block opened early that uses a node declared for a
        later block), without it: one region, every node in topological order."""
        try:
            return self._part(terms, outer_regs, skip=True)
        except _OrderError:
            return self._part(terms, outer_regs, skip=False)
        finally:
            self._order = None

    def _part(self, terms: Sequence[Tuple[int, int]], outer_regs: bool, skip: bool) -> str:
        """Body of one part function: every (node, output) term OR-ed into the warp's
        shared-memory accumulator of its output.

        Zero-block skipping by guard regions.  A checkpoint is an AND on a marker path (1st AND,
        then every `skip_interval` ANDs, counting restarts after an addition).  cz(v) is the set
        of checkpoints whose being zero in the whole tile makes v zero in its exact lanes:
        AND/Advance inherit the union of their marker operands' sets, OR/XOR/SEL the
        intersection, everything else nothing.  v is computed inside the guard of the latest
        checkpoint in cz(v) other than itself (its home); a value used outside its home is
        declared zero in the enclosing region both share.  Within a region the unguarded work
        is emitted first and child guard blocks are opened as late as dependencies allow, so
        the dense part of all terms forms one basic block.

        With `outer_regs` every term ORs into register accumulators `oa<o>_<j>` that the
        caller declares and stores (the split form's parts)."""
        d = self.d
        k = max(1, self.t.skip_interval) if self.t.skip_interval > 0 and skip else 0
        self.lines = []
        self.indent = 2
        self.scopes = [{}]
        term_outs: Dict[int, List[int]] = {}
        for v, o in terms:
            term_outs.setdefault(v, []).append(o)
        # outputs with several terms here OR them in registers and reach the shared-memory
        # accumulator once, at the end of the part (a term costs one OR instead of a vote,
        # a load and a store)
        n_terms: Dict[int, int] = {}
        for _, o in terms:
            n_terms[o] = n_terms.get(o, 0) + 1
        reg_out = sorted(o for o, c in n_terms.items() if c > 1 or outer_regs)
        if not outer_regs:
            for o in reg_out:
                self.declare_zero(f"oa{o}")
        # heavy nodes of this part, in topological (id) order
        heavy = sorted(set().union(*[self.heavy_ancestors(v) for v in term_outs]))
        hs = set(heavy)
        computed: set = set()
        lifted: set = set()
        self._order = (hs, computed, lifted)   # see mat()
        andd: Dict[int, int] = {}
        cz: Dict[int, frozenset] = {}
        ckpt = set()
        # late = needs the result of an addition; additions are split so that their carry
        # look-back is issued after all early work of the part
        late: Dict[int, bool] = {}
        late_in: Dict[int, bool] = {}
        for v in heavy:
            n = d.nodes[v]
            ha = [a for a in n.args if a in hs]
            late_in[v] = any(late[a] for a in ha)
            deferred = n.op in ADD_OPS and self.wide_class(n.args[1]) and v not in self.pre
            late[v] = deferred or late_in[v]
        for v in heavy:
            n = d.nodes[v]
            ha = [a for a in n.args if a in hs]
            if n.op in ADD_OPS:
                andd[v] = 0
                cz[v] = frozenset()
                continue
            andd[v] = max([andd[a] for a in ha] + [0]) + (1 if n.op == "and" else 0)
            if n.op == "and":
                c = frozenset().union(*[cz[a] for a in ha]) if ha else frozenset()
                if k and andd[v] >= 1 and (andd[v] - 1) % k == 0:
                    ckpt.add(v)
                    c = c | {v}
            elif n.op in ("advance", "lookahead"):
                c = cz[ha[0]] if ha else frozenset()
            elif n.op in ("or", "xor"):
                c = cz[ha[0]] & cz[ha[1]] if len(ha) == 2 else frozenset()
            elif n.op == "sel":
                a1, a2 = n.args[1], n.args[2]
                c = (cz[a1] if a1 in hs else frozenset()) & (cz[a2] if a2 in hs else frozenset()) \
                    if (a1 in hs and a2 in hs) else frozenset()
            else:
                c = frozenset()
            if late[v]:  # late work only runs inside late guards, so regions never mix
                c = frozenset(z for z in c if late[z])
            cz[v] = c
        TOP = -1
        home: Dict[int, int] = {}
        for v in heavy:
            c = cz[v] - {v}
            home[v] = max(c) if c else TOP
        parent = {z: home[z] for z in ckpt}

        def chain(r):  # regions from r up to TOP
            out = [r]
            while r != TOP:
                r = parent[r]
                out.append(r)
            return out

        def lca(a, b):
            ca = chain(a)
            sb = set(chain(b))
            for r in ca:
                if r in sb:
                    return r
            return TOP

        users: Dict[int, List[int]] = {v: [] for v in heavy}
        for v in heavy:
            for a in d.nodes[v].args:
                if a in hs:
                    users[a].append(v)
        decl: Dict[int, int] = {}
        for v in heavy:
            r = home[v]
            for u in users[v]:
                r = lca(r, home[u])
            decl[v] = r
        by_home: Dict[int, List[int]] = {}
        for v in heavy:
            by_home.setdefault(home[v], []).append(v)
        lifted_at: Dict[int, List[int]] = {}
        for v in heavy:
            if decl[v] != home[v]:
                lifted_at.setdefault(decl[v], []).append(v)
        children: Dict[int, List[int]] = {}
        for z in sorted(ckpt):
            children.setdefault(parent[z], []).append(z)

        def child_of(R, r):
            """The child region of R on the path to region r, or None."""
            prev = None
            while r != R:
                if r == TOP:
                    return None
                prev = r
                r = parent[r]
            return prev

        begun = set()

        def add_begin(v):
            n = d.nodes[v]
            m, c = self.mat(n.args[0]), self.mat(n.args[1])
            mode = 0 if n.op == "matchstar" else 1
            fn = "add_known" if v in self.pre else "add_begin"
            self.emit(f"const AddState st{v} = {fn}<{self.dl[v]}, E>(p, t, {self.adds[v]}, {mode}, "
                      f"{self.pack(m)}, {self.pack(c)});")
            begun.add(v)

        def compute(v):
            n = d.nodes[v]
            name = f"v{v}"
            declare = decl[v] == home[v]
            self.epoch = self.epochs.get(v, -1)
            if n.op in ADD_OPS:
                if v not in begun:
                    add_begin(v)
                m, c = self.mat(n.args[0]), self.mat(n.args[1])
                mode = 0 if n.op == "matchstar" else 1
                self.emit(f"const S {name}_s = add_end<{self.dl[v]}, E>(p, t, {self.adds[v]}, {mode}, st{v}, "
                          f"{self.pack(m)}, {self.pack(c)});")
                for j in range(self.t.wpt):
                    pre = "const uint32_t " if declare else ""
                    self.emit(f"{pre}{name}_{j} = {name}_s.w[{j}];")
            else:
                a = [self.operand(x) if n.op in ("and", "or", "xor") else self.mat(x)
                     for x in n.args]
                self.emit_op(name, n, a, declare=declare)
            self.scopes[-1][v] = name
            computed.add(v)
            if declare is False:
                self.scopes[0][v] = name  # visible everywhere below its declaration
            for o in term_outs.get(v, []):
                if o in reg_out:
                    for j in range(self.t.wpt):
                        self.emit(f"oa{o}_{j} |= {name}_{j};")
                else:
                    self.emit(f"acc_or(acc, {o}, {self.pack(name)});")

        def emit_top():
            for v in lifted_at.get(TOP, []):
                self.emit("uint32_t " + ", ".join(f"v{v}_{j} = 0u" for j in range(self.t.wpt)) + ";")
                self.scopes[-1][v] = f"v{v}"
                lifted.add(v)
            kids = children.get(TOP, [])
            done_children = set()
            for phase in (1, 2):
                ready: List[int] = []
                for v in by_home.get(TOP, []):
                    is_add = d.nodes[v].op in ADD_OPS
                    if phase == 1:
                        if late_in[v]:
                            continue
                        if not is_add and late[v]:
                            continue
                    else:
                        if not late[v]:
                            continue
                    for a in d.nodes[v].args:
                        if a in hs and home[a] != TOP:
                            c = child_of(TOP, home[a])
                            if c is not None and c not in done_children:
                                emit_child(c)
                                done_children.add(c)
                                if c in ready:
                                    ready.remove(c)
                    if phase == 1 and is_add and late[v]:
                        add_begin(v)      # deferred: the look-back is issued in phase 2
                        continue
                    compute(v)
                    if v in kids:
                        ready.append(v)
                        while len(ready) > self.t.window:
                            c = ready.pop(0)
                            emit_child(c)
                            done_children.add(c)
                for c in sorted(kids):
                    if c not in done_children and (phase == 2 or not late[c]):
                        emit_child(c)
                        done_children.add(c)

        def emit_region(R):
            for v in lifted_at.get(R, []):
                self.emit("uint32_t " + ", ".join(f"v{v}_{j} = 0u" for j in range(self.t.wpt)) + ";")
                self.scopes[-1][v] = f"v{v}"
                lifted.add(v)
            kids = set(children.get(R, []))
            ready: List[int] = []          # computed checkpoints whose block is not emitted yet
            done_children = set()
            for v in by_home.get(R, []):
                for a in d.nodes[v].args:
                    if a in hs and home[a] != R:
                        c = child_of(R, home[a])
                        if c is not None and c not in done_children:
                            emit_child(c)
                            done_children.add(c)
                            if c in ready:
                                ready.remove(c)
                compute(v)
                if v in kids:
                    ready.append(v)
                    while len(ready) > self.t.window:
                        c = ready.pop(0)
                        emit_child(c)
                        done_children.add(c)
            for c in sorted(kids):
                if c not in done_children:
                    emit_child(c)
                    done_children.add(c)

        def emit_child(z):
            self.open(self.any_expr(f"v{z}"))
            emit_region(z)
            self.close()

        emit_top()
        # terms that are pure character classes (no heavy node)
        for v, os_ in term_outs.items():
            if v not in hs:
                r = self.mat(v)
                if r != "0u":
                    for o in os_:
                        if o in reg_out:
                            for j in range(self.t.wpt):
                                self.emit(f"oa{o}_{j} |= {self.w(r, j)};")
                        else:
                            self.emit(f"acc_or(acc, {o}, {self.pack(r)});")
        if not outer_regs:
            for o in reg_out:
                self.emit(f"acc_or(acc, {o}, {self.pack(f'oa{o}')});")
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


SMEM_BUDGET = 48 * 1024
WCOUNT_MAX = 64    # split-form programs with at most this many outputs keep match counts per warp
# Passes that visit every tile once without waiting take chunks of 32 consecutive tiles per warp,
# so that each pre-pass addition's aggregate bits of a chunk fill one word (pre_collect/flush).
_CHUNK_HEAD = (
    "  const long long rows = (p.n_tiles + 31) >> 5;\n"
    "  /* chunks of CT consecutive tiles (1..32, a power of two, so a chunk stays in one row of\n"
    "     32 tiles): small launches use short chunks, so that every warp has work */\n"
    "  const int CT = p.chunk_tiles > 0 ? p.chunk_tiles : 32;\n"
    "  const long long chunks = (p.n_tiles + CT - 1) / CT;\n"
    "  const long long stride = (long long)gridDim.x * (blockDim.x >> 5);\n"
    "  for (long long c = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); c < chunks; c += stride) {\n"
    "   const long long g0 = c * CT, g1 = g0 + CT < p.n_tiles ? g0 + CT : p.n_tiles, row = g0 >> 5;\n"
    "   const int l0 = (int)(g0 & 31);\n"
    "   uint32_t gw[NPRE_WORDS], pw[NPRE_WORDS];\n"
    "   for (int j = 0; j < NPRE_WORDS; ++j) gw[j] = pw[j] = 0u;\n")
_TILE_LOOP = (
    "   for (int l = l0; l < l0 + CT; ++l) {\n"
    "    const long long g = row * 32 + l;\n"
    "    if (g >= p.n_tiles) break;\n"
    "    uint32_t pg[NPRE_WORDS], pp[NPRE_WORDS];\n"
    "    for (int j = 0; j < NPRE_WORDS; ++j) pg[j] = pp[j] = 0u;\n")
PRE_CHUNK_OPEN = _CHUNK_HEAD + _TILE_LOOP
CLS_CHUNK_OPEN = (                   # classify: PRE_CHUNK_OPEN plus the chunk's output zeroing
    _CHUNK_HEAD +
    "   const int zin = chunk_input(p, g0, g1);\n"
    "   /* a chunk inside one input: its first tile and length, for every tile's setup */\n"
    "   const long long zfirst = zin >= 0 ? p.tile_prefix[zin] : 0, zn = zin >= 0 ? p.in_len[zin] : 0;\n"
    "   if (zin >= 0) { @ZERO@ }\n"
    "   cx.row = row;\n"
    "   bool pf = false;\n"
    "   uint32_t nraw[BG_WPT][8];\n" + _TILE_LOOP)
CLS_CHUNK_CLOSE = (
    "    if (NPRE > 0) pre_collect(pg, pp, gw, pw, l, t.lane);\n"
    "   }\n"
    "@CHUNKEND@"
    "   if (NPRE > 0) pre_flush(p, row, gw, pw, t.lane, CT < 32);\n"
    "   flush_runs(p, row, l0, CT, runs_s, @ROWRUN@, t.lane);\n"
    "  }\n")
PRE_CHUNK_CLOSE = (
    "    if (NPRE > 0) pre_collect(pg, pp, gw, pw, l, t.lane);\n"
    "   }\n"
    "   if (NPRE > 0) pre_flush(p, row, gw, pw, t.lane, CT < 32);\n"
    "  }\n")

def _cluster_terms(gen: "_Gen", terms: List[Tuple[int, int]], cap: int) -> List[List[Tuple[int, int]]]:
    """Union terms that share a non-character-class node (a common prefix chain, an addition),
    so that shared work is done once per tile; clusters hold at most `cap` terms."""
    parent = list(range(len(terms)))
    size = [1] * len(terms)

    def find(i):
        while parent[i] != i:
            parent[i] = parent[parent[i]]
            i = parent[i]
        return i

    owner: Dict[int, int] = {}
    for i, (v, _) in enumerate(terms):
        for h in sorted(gen.heavy_ancestors(v)):
            if h in owner:
                a, b = find(i), find(owner[h])
                if a != b and size[a] + size[b] <= cap:
                    if size[a] < size[b]:
                        a, b = b, a
                    parent[b] = a
                    size[a] += size[b]
            else:
                owner[h] = i
    groups: Dict[int, List[Tuple[int, int]]] = {}
    for i, t in enumerate(terms):
        groups.setdefault(find(i), []).append(t)
    # pack small clusters together so there are few, mid-sized functions
    out: List[List[Tuple[int, int]]] = []
    cur: List[Tuple[int, int]] = []
    for g in sorted(groups.values(), key=len, reverse=True):
        if cur and len(cur) + len(g) > cap:
            out.append(cur)
            cur = []
        cur = cur + g
    if cur:
        out.append(cur)
    return out


def generate_kernel(groups: Sequence[Group], tuning: Optional[Tuning] = None,
                    per_regex: bool = False, name: str = "bg_scan") -> KernelSpec:
    """Lower the pattern set into one kernel.

    All groups share one hash-consed DAG.  Its outputs are split into OR-ed terms, and terms that
    share work (a common literal prefix, the same addition) are clustered into non-inlined part
    functions (compile time grows linearly with the pattern set; NVRTC can split the work).
    Each part ORs its terms into per-warp shared-memory accumulators, one per output; after all
    parts ran on a tile, the accumulators are written out.  Output grouping is therefore
    independent of how the computation is partitioned."""
    tuning = tuning or Tuning()
    wpt = tuning.wpt
    dag, outs, names = build_dag(groups, per_regex)
    gen = _Gen(dag, tuning)
    gen.analyse(outs)
    n_out = len(outs)
    terms: List[Tuple[int, int]] = []
    for o, v in enumerate(outs):
        for leaf in gen.or_leaves(v):
            terms.append((leaf, o))
    filt = None
    if tuning.prefilter and not tuning.lockstep and not tuning.edge_variants:
        pre_nodes = [v for v, _ in sorted(gen.pre.items(), key=lambda x: x[1])]
        filt = prefilter.build(gen, [v for v, _ in terms], pre_nodes,
                               config=tuning.filter_config, bloom_bits=tuning.bloom_bits)
        positions = 32 * 32 * tuning.wpt
        lim = tuning.prefilter_limit
        if not filt.enabled or (lim < 1.0 and (
                filt.expected_per_tile(positions) > lim * len(terms)
                or filt.hits * 1024 / positions > lim * 8)):
            # the filter would pass most terms: single-kernel form, with its own tile shape
            # (programs whose terms have no filter at all keep the requested shape)
            # (the terms run on every tile and mostly stay non-zero for several steps, so
            # zero-block skipping costs more branches than it saves: off by default)
            if filt.enabled and tuning.single_wpt and (tuning.single_wpt != tuning.wpt or
                                                        tuning.single_min_blocks != tuning.min_blocks or
                                                        tuning.single_edge != tuning.edge_variants):
                return generate_kernel(groups, replace(
                    tuning, prefilter=False, wpt=tuning.single_wpt,
                    min_blocks=tuning.single_min_blocks, edge_variants=tuning.single_edge,
                    skip_interval=0 if tuning.skip_interval < 0 else tuning.skip_interval),
                    per_regex, name)
            if filt.enabled and tuning.skip_interval < 0:
                tuning = replace(tuning, skip_interval=0)
                gen.t = tuning
            filt = None
    if tuning.skip_interval < 0:
        tuning = replace(tuning, skip_interval=0 if filt is not None else 1)
        gen.t = tuning
    if filt is not None:
        if tuning.exec_min_blocks:
            tuning = replace(tuning, min_blocks=tuning.exec_min_blocks)
            gen.t = tuning
        return _generate_filtered(gen, tuning, terms, names, filt, name)
    if tuning.push_advances:
        outs = push_advances(dag, outs)
        epochs: Dict[int, int] = {}
        if tuning.chain_batch > 0:
            outs, epochs = interleave_chains(dag, outs, tuning.chain_batch, tuning.pair_share)
        gen = _Gen(dag, tuning)
        gen.analyse(outs)
        gen.share_reads = True
        gen.epochs = epochs
        terms = [(leaf, o) for o, v in enumerate(outs) for leaf in gen.or_leaves(v)]
    budget = SMEM_BUDGET
    per_warp = max(1, n_out) * wpt * 32 * 4
    if per_warp > budget:
        raise NotFusable(f"{n_out} outputs need {per_warp} bytes of accumulators per warp; "
                         f"use fewer outputs per program")
    if (tuning.block // 32) * per_warp > budget:
        # many outputs: fewer warps per block keep the accumulators within the budget
        block = max(32, (budget // per_warp) * 32)
        tuning = replace(tuning, block=block,
                         min_blocks=min(32, -(-tuning.min_blocks * tuning.block // block)))
    warps = tuning.block // 32
    clusters = _cluster_terms(gen, terms, tuning.part_cap or 64)
    funcs = []
    sig = f"const BgParams &p, const Tile &t, uint32_t *acc, {_basis_params(wpt)}"
    args = f"p, t, acc, {', '.join(f'b{i}_{j}' for i in range(8) for j in range(wpt))}"
    for ci, cl in enumerate(clusters):
        code = gen.part(cl)
        # E = the tile touches an input boundary: only then are the start/end masks applied
        fast = (f'extern "C" __device__ __noinline__ void bg_part_{ci}_0({sig}) {{ bg_part_{ci}_body<false>({args}); }}\n'
                if tuning.edge_variants else "")
        funcs.append(
            f"//@@BG_PART\n"
            f"template <bool E> __device__ __forceinline__ void bg_part_{ci}_body({sig}) {{\n{code}\n}}\n"
            + fast +
            f'extern "C" __device__ __noinline__ void bg_part_{ci}_1({sig}) {{ bg_part_{ci}_body<true>({args}); }}\n')
    decls = "\n".join(
        f'extern "C" __device__ void bg_part_{ci}_{e}({sig});'
        for ci in range(len(clusters)) for e in ((0, 1) if tuning.edge_variants else (1,)))
    ba = _basis_args(wpt)
    if tuning.edge_variants:
        calls = ("    if (t.edge) {\n"
                 + "\n".join(f"      bg_part_{ci}_1(p, t, acc, {ba});" for ci in range(len(clusters)))
                 + "\n    } else {\n"
                 + "\n".join(f"      bg_part_{ci}_0(p, t, acc, {ba});" for ci in range(len(clusters)))
                 + "\n    }")
    else:
        calls = "\n".join(f"    bg_part_{ci}_1(p, t, acc, {ba});" for ci in range(len(clusters)))
    comments = "\n".join(f"/* output {o}: {nm.replace('*/', '* /')} */" for o, nm in enumerate(names))
    # (the single-kernel form adds each tile's counts directly: a count cache measured slower
    # there, its registers being taken by the terms)
    wcount = 0
    counts_begin = (f"  __shared__ unsigned long long bg_cnt_s[{warps} * {max(1, wcount)}];\n"
                    f"  if (BG_WCOUNT > 0) count_cache_begin(t, bg_cnt_s + (threadIdx.x >> 5) * BG_WCOUNT);\n")
    kernel_free = (
        f"  __shared__ uint32_t bg_acc[{warps} * BG_NOUT * BG_WPT * 32];\n"
        f"  uint32_t *acc = bg_acc + (threadIdx.x >> 5) * (BG_NOUT * BG_WPT * 32);\n"
        f"  Tile t;\n"
        f"  init(p, t);\n"
        + counts_begin +
        f"  while (next_tile(p, t)) {{\n"
        f"    acc_clear(acc, t);\n"
        f"    S b[8];\n"
        f"    load_basis(p, t, b);\n"
        f"{calls}\n"
        f"    acc_store(p, t, acc);\n"
        f"  }}\n"
        f"  flush_counts(p, t);\n"
        f"}}\n")
    lock_calls = "\n".join(f"    if (has) bg_part_{ci}_1(p, t, acc, {ba});\n    __syncthreads();"
                            for ci in range(len(clusters)))
    kernel_lockstep = (
        f"  __shared__ uint32_t bg_acc[{warps} * BG_NOUT * BG_WPT * 32];\n"
        f"  __shared__ unsigned int bg_claim;\n"
        f"  uint32_t *acc = bg_acc + (threadIdx.x >> 5) * (BG_NOUT * BG_WPT * 32);\n"
        f"  Tile t;\n"
        f"  init(p, t);\n"
        + counts_begin +
        f"  for (;;) {{\n"
        f"    const unsigned int g0 = claim_block(p, &bg_claim);\n"
        f"    if ((long long)g0 >= p.n_tiles) break;\n"
        f"    const unsigned int g = g0 + (threadIdx.x >> 5);\n"
        f"    const bool has = (long long)g < p.n_tiles;\n"
        f"    S b[8];\n"
        f"    if (has) {{ setup_tile(p, t, g); acc_clear(acc, t); load_basis(p, t, b); }}\n"
        f"{lock_calls}\n"
        f"    if (has) acc_store(p, t, acc);\n"
        f"  }}\n"
        f"  flush_counts(p, t);\n"
        f"}}\n")
    # registers a thread may use so that min_blocks blocks fit: each of the SM's four
    # sub-partitions holds 16K registers for its share of the resident warps
    warps_per_smsp = -(-(tuning.block // 32) * max(1, tuning.min_blocks) // 4)
    maxreg = max(32, min(255, (16384 // (warps_per_smsp * 32)) // 8 * 8))
    pre_kernel = ""
    if gen.pre:
        basis_decl = ", ".join(f"b{i}_{j} = b[{i}].w[{j}]" for i in range(8) for j in range(wpt))
        pre_kernel = (
            f"//@@BG_PART\n"
            f"/* carry pre-pass: the aggregates of additions 0..{len(gen.pre) - 1} for every tile, no waits;\n"
            f"   tiles are taken in a fixed stride since nothing here waits on another tile */\n"
            f'extern "C" __global__ void __launch_bounds__({tuning.block}, {tuning.min_blocks}) {name}_pre(const __grid_constant__ BgParams p) {{\n'
            f"  Tile t;\n"
            f"  init(p, t);\n"
            f"{PRE_CHUNK_OPEN}"
            f"    setup_tile(p, t, (unsigned int)g, false, false);\n"
            f"    S b[8];\n"
            f"    load_basis(p, t, b);\n"
            f"    const uint32_t {basis_decl};\n"
            f"    constexpr bool E = true;\n"
            f"{gen.pre_body()}\n"
            f"{PRE_CHUNK_CLOSE}"
            f"}}\n")
    src = (
        f"//@@BG_MAXREG {maxreg}\n"
        f"#define BG_WPT {wpt}\n"
        f"#define BG_HL {gen.hl}\n"
        f"#define BG_TL {gen.tl}\n"
        f"#define BG_NOUT {n_out}\n"
        f"#define BG_WCOUNT {wcount}\n"
        f"#define BG_CLAIM_TILES {max(1, tuning.claim_tiles)}\n"
        f"#define BG_LOOKBACK_INLINE {int(tuning.inline_lookback)}\n"
        f"#define BG_LBK {tuning.lookback_width}\n"
        f"#define BG_LB_SPIN {tuning.lookback_spin}\n"
        f"#define BG_NPRE {len(gen.pre)}\n"
        f'#include "bg_device.cuh"\n'
        f"using namespace bg;\n"
        f"#define VM(j) (E ? t.vm.w[j] : 0xffffffffu)\n"
        f"#define EM(j) (E ? t.em.w[j] : 0xffffffffu)\n"
        f"{comments}\n"
        + "\n".join(funcs) + pre_kernel +
        f"//@@BG_KERNEL\n{decls}\n"
        f'extern "C" __global__ void __launch_bounds__({tuning.block}, {tuning.min_blocks}) {name}(const __grid_constant__ BgParams p) {{\n'
        + (kernel_lockstep if tuning.lockstep else kernel_free)
    )
    return KernelSpec(source=src, name=name, n_outputs=n_out, n_adds=len(gen.adds),
                      halo_lanes=gen.hl, wpt=wpt, block=tuning.block, max_depth_bits=gen.max_dbits,
                      n_nodes=len(dag.nodes), output_names=names, tail_lanes=gen.tl,
                      n_pre=len(gen.pre))


def _hex_array(vals: Sequence[int], per_line: int = 12) -> str:
    lines = []
    for i in range(0, len(vals), per_line):
        lines.append("  " + ", ".join(f"0x{v:08x}u" for v in vals[i:i + per_line]) + ",")
    return "\n".join(lines)


def _generate_filtered(gen: "_Gen", tuning: Tuning, terms: List[Tuple[int, int]],
                       names: List[str], filt: "prefilter.TermFilter", name: str) -> KernelSpec:
    """The split, prefiltered form of the program: two kernels.

    ``<name>_cls`` (classify) visits every tile once, with nothing to wait for: it scans the
    tile's q-grams (bg_device.cuh load_scan), publishes the carry pre-pass aggregates, adds the
    terms whose look-back additions could take or owe a carry (class all ones at the carry lane
    or at the successor's) and those whose filter holds only through a pre-pass carry, and
    writes the tile's run mask (one bit per term) to ``p.runs``.

    ``<name>`` (execute) runs after the carry scan and the runtime's work-list kernel.  Its work
    items are (part, row of 32 tiles) pairs where the part has work.  Part k belongs to SM group
    k % exec_groups; the warps of an SM claim their group's items (part-major, rows increasing)
    from the group's counter, then help the other groups, so an SM keeps few part bodies in its
    instruction caches.  A warp reads the row's 32 run masks with one load, and for each tile
    where one of the part's terms runs it loads the basis and calls the part, which ORs its
    terms into per-warp accumulators and merges them into the outputs (atomicOr over the zeros
    classify wrote, counting only newly set bits) or, without merging, stores whole outputs.
    Tiles of one part are claimed in increasing order, which keeps the look-back of its
    additions deadlock free."""
    d = gen.d
    wpt = tuning.wpt
    warps = tuning.block // 32
    nt = len(terms)
    nw = filt.words
    always = filt.always_mask()
    for r, cond in enumerate(filt.term_cond):
        if cond:                       # classify runs before the carry scan: no carry-ins yet
            always |= 1 << r
    sl = 32 - gen.hl - gen.tl
    # look-back obligations -----------------------------------------------------------------
    pm_classes: Dict[int, str] = {}
    need_masks: Dict[Tuple[int, int], int] = {}   # (class, carry lane) -> terms to run
    needs: List[bool] = [False] * nt
    for r, (v, _) in enumerate(terms):
        if (always >> r) & 1:
            continue
        for a in sorted(gen.heavy_ancestors(v)):
            n = d.nodes[a]
            if n.op not in ADD_OPS or a in gen.pre:
                continue
            c = n.args[1]
            if not d.is_cc(c):
                always |= 1 << r
                break
            pm_classes.setdefault(c, f"pm{c}")
            key = (c, gen.dl[a])
            need_masks[key] = need_masks.get(key, 0) | (1 << r)
            needs[r] = True
    # parts of whole outputs ----------------------------------------------------------------
    by_out: Dict[int, List[int]] = {}
    for r, (v, o) in enumerate(terms):
        by_out.setdefault(o, []).append(r)
    cap = max(1, tuning.part_cap or 2)
    merge = tuning.merge_outputs
    part_terms: List[List[int]] = []     # terms of each part, in output order
    if merge:
        order = [r for o in range(len(names)) for r in by_out.get(o, [])]
        part_terms = [order[i:i + cap] for i in range(0, len(order), cap)]
    else:                                # whole outputs per part
        cur: List[int] = []
        n_outs = 0
        for o in range(len(names)):
            rs = by_out.get(o, [])
            if cur and (len(cur) + len(rs) > cap or n_outs >= 32):
                part_terms.append(cur)
                cur, n_outs = [], 0
            cur = cur + rs
            n_outs += 1
        if cur:
            part_terms.append(cur)
    parts: List[List[int]] = []          # outputs of each part
    for rs in part_terms:
        outs_k: List[int] = []
        for r in rs:
            if terms[r][1] not in outs_k:
                outs_k.append(terms[r][1])
        parts.append(outs_k)
    nacc = max(1, max(len(ps) for ps in parts))
    sig = f"const BgParams &p, const Tile &t, uint32_t *acc, {_basis_params(wpt)}"
    funcs = []
    part_masks: List[Dict[int, int]] = []
    # a part receives the tile's run words it tests as r0, r1, ... (its words in increasing order)
    pmw = max(1, max(len({r >> 5 for r in rs}) for rs in part_terms))
    sig = (f"const BgParams &p, const Tile &t, uint32_t *acc, "
           + "".join(f"uint32_t r{i}, " for i in range(pmw)) + _basis_params(wpt))
    for ci, (rs, outs_k) in enumerate(zip(part_terms, parts)):
        blocks = []
        masks: Dict[int, int] = {}
        for r in rs:
            masks[r >> 5] = masks.get(r >> 5, 0) | (1 << (r & 31))
        words = sorted(masks)
        for r in rs:
            li = outs_k.index(terms[r][1])
            code = gen.part([(terms[r][0], li)], outer_regs=True)
            body = "\n".join("  " + ln for ln in code.split("\n"))
            blocks.append(f"  if ((r{words.index(r >> 5)} >> {r & 31}) & 1u) {{\n{body}\n  }}")
        part_masks.append(masks)
        fn = "merge_store" if merge else "store"
        # the terms OR into register accumulators, one per output of the part
        regs = "\n".join(f"  uint32_t " + ", ".join(f"oa{li}_{j} = 0u" for j in range(wpt)) + ";"
                         for li in range(len(outs_k)))
        stores = "\n".join(f"  {fn}(p, t, {o}, {gen.pack(f'oa{li}')});" for li, o in enumerate(outs_k))
        funcs.append(f"{{PART}}"
                     f'{{QUAL}} void bg_part_{ci}({sig}) {{\n'
                     f"  constexpr bool E = true;\n"
                     f"{regs}\n" + "\n".join(blocks) + "\n" + stores + "\n}\n")
    # up to inline_parts parts are inlined into the execute kernel (one translation unit, no call
    # per tile: the call would save the item loop's registers and pass the tile by memory);
    # more parts are separate translation units compiled in parallel and called through a table
    inline = 0 < len(parts) <= tuning.inline_parts
    if inline:
        # one whole-program compile of classify and execute (two sections): relocatable code
        # measured slower for the inlined kernel
        funcs = ["".join(f.replace("{PART}", "").replace("{QUAL}", "static __device__ __forceinline__")
                         for f in funcs)]
        decls = ""
    else:
        funcs = [f.replace("{PART}", "//@@BG_PART\n").replace("{QUAL}", 'extern "C" __device__ __noinline__')
                 for f in funcs]
        decls = "\n".join(f'extern "C" __device__ void bg_part_{ci}({sig});' for ci in range(len(parts)))
    # execute order: part k belongs to group k % ngroups; groups one after the other
    ngroups = max(1, min(16, tuning.exec_groups, len(parts)))
    ord_ = [k for gi in range(ngroups) for k in range(gi, len(parts), ngroups)]
    gpos = [0]
    for gi in range(ngroups):
        gpos.append(gpos[-1] + len(range(gi, len(parts), ngroups)))
    decls += (f"\n__constant__ int bg_ord[{len(parts)}] = {{{', '.join(map(str, ord_))}}};"
              f"\n__constant__ int bg_gpos[{ngroups + 1}] = {{{', '.join(map(str, gpos))}}};")
    ba = ", ".join(f"b[{i}].w[{j}]" for i in range(8) for j in range(wpt))
    pmw = max(1, max(len(m) for m in part_masks))
    pm_table = []
    for masks in part_masks:
        items_ = sorted(masks.items()) + [(0, 0)] * (pmw - len(masks))
        for w, m in items_:
            pm_table += [w, m]
    # execute dispatch: the parts' (run word, mask) pairs in shared memory and a table of the
    # part functions, so that one call site serves every part
    fn_tab = ((f"typedef void (*bg_part_fn)({sig});\n"
               f"__device__ bg_part_fn bg_part_tab[{len(parts)}] = {{{', '.join(f'bg_part_{ci}' for ci in range(len(parts)))}}};\n")
              if not inline else "") + f'extern "C" __device__ const uint32_t bg_pmask[{len(pm_table)}];\n'
    part_args = f"p, t, acc, {''.join(f'__shfl_sync(FULL, rw{i}, l), ' for i in range(pmw))}{ba}"
    if inline:
        dispatch = ("      switch (k) {\n" + "".join(f"        case {ci}: bg_part_{ci}({part_args}); break;\n"
                                                 for ci in range(len(parts)))
                    + "        default: break;\n      }\n")
    else:
        dispatch = f"      bg_part_tab[k]({part_args});\n"
    # classify kernel ------------------------------------------------------------------------
    # The tile's bytes are at hand (raw); its basis planes are made only where a class test
    # needs them (basis_of): a class whose complement is at most three bytes (such as '.',
    # everything but a line feed) is tested on the bytes themselves, and the branches that
    # compute classes from the basis run on few tiles.
    gen.lines = []
    gen.indent = 4
    gen.scopes = [{}]
    basis_decl = ", ".join(f"b{i}_{j} = bb[{i}].w[{j}]" for i in range(8) for j in range(wpt))
    basis_block = f"S bb[8]; basis_of(raw, bb); const uint32_t {basis_decl};"
    # the terms that always run start every tile's run words (bg_always, preset by load_scan)
    always_words = [(always >> (32 * w)) & 0xFFFFFFFF for w in range(nw)]
    # pre-pass aggregates: with a zero marker (no q-gram of it in the tile) the aggregate
    # depends on the class alone
    # additions sharing a class and carry lane have the same zero-marker aggregate: one test
    # per group; an addition whose marker filter fired (rare) replaces its bits
    groups_: Dict[Tuple[int, int], int] = {}
    for v, k in gen.pre.items():
        key = (d.nodes[v].args[1], gen.dl[v])
        groups_[key] = groups_.get(key, 0) | (1 << k)
    full256 = (1 << 256) - 1

    def excluded(cnode):
        """The bytes outside class `cnode` when there are one to three of them, else None (also
        when the addition runs over a stream that is not a class, e.g. shifted classes)."""
        if not d.is_cc(cnode):
            return None
        comp = ~gen.byteset(cnode) & full256
        xs = [b for b in range(256) if (comp >> b) & 1]
        return xs if 1 <= len(xs) <= 3 else None
    basis_always = any(excluded(c) is None for (c, _) in groups_)
    if basis_always:
        gen.emit(basis_block)
    for (cnode, dl), kmask in sorted(groups_.items()):
        xs = excluded(cnode)
        if xs is not None:
            args = ", ".join(f"{x}u" for x in xs)
            gen.emit(f"{{ const uint32_t pz = pre_propagates<{dl}>(excl_lanes<{len(xs)}, {args}>(t, raw)) ? 0xffffffffu : 0u;")
        else:
            c = gen.mat(cnode)
            gen.emit(f"{{ const uint32_t pz = pre_propagates<{dl}>(ones_lanes(t, {gen.pack(c)})) ? 0xffffffffu : 0u;")
        for j in range(-(-len(gen.pre) // 32)):
            m = (kmask >> (32 * j)) & 0xFFFFFFFF
            if m:
                gen.emit(f"  pp[{j}] |= pz & 0x{m:08x}u;")
        gen.emit("}")
    # additions whose marker filter fired (a few percent of tiles): out of line, one function per
    # word of 32 additions, so that the common path stays short in the instruction caches
    cand_funcs = []
    cand_calls = []
    saved = (gen.lines, gen.indent, gen.scopes)
    pre_sorted = sorted(gen.pre.items(), key=lambda x: x[1])
    for j in range(-(-len(gen.pre) // 32)):
        gen.lines, gen.indent, gen.scopes = [], 2, [{}]
        run_bits: Dict[int, int] = {}
        for v, k in pre_sorted:
            if k >> 5 != j:
                continue
            n = d.nodes[v]
            bit = nt + k
            run_bits[bit >> 5] = run_bits.get(bit >> 5, 0) | (1 << (bit & 31))
            mode = 0 if n.op == "matchstar" else 1
            gen.open(f"(run[{32 * (bit >> 5)}] >> {bit & 31}) & 1u")
            m = gen.mat(n.args[0])
            c = gen.mat(n.args[1])
            gen.emit(f"uint32_t G, P; pre_aggregate<{gen.dl[v]}, E>(t, {mode}, {gen.pack(m)}, {gen.pack(c)}, G, P); "
                     f"pg |= G << {k & 31}; pm |= 1u << {k & 31}; pv |= P << {k & 31};")
            gen.close()
        cand_funcs.append(
            f"static __device__ __noinline__ uint3 bg_cand_{j}(const Tile &t, const uint32_t *run, {_basis_params(wpt)}) {{\n"
            f"  constexpr bool E = true;\n"
            f"  uint32_t pg = 0u, pm = 0u, pv = 0u;\n" + "\n".join(gen.lines) + "\n"
            f"  return make_uint3(pg, pm, pv);\n}}\n")
        # at the chunk's end, once its Bloom hits are resolved: lane i looks at tile l0 + i,
        # and every tile where the marker filter of one of these additions fired gets their
        # aggregates from its basis, replacing the zero-marker bits pre_collect gathered
        cond = " | ".join(f"(runs_s[{32 * w} + l0 + t.lane] & 0x{m:08x}u)" for w, m in sorted(run_bits.items()))
        basis_names = ", ".join(f"b{i}_{jj}" for i in range(8) for jj in range(wpt))
        cand_calls.append(
            f"   {{ const uint32_t cw = (t.lane < CT && row * 32 + l0 + t.lane < p.n_tiles) ? ({cond}) : 0u;\n"
            f"     for (uint32_t todo = __ballot_sync(FULL, cw != 0u); todo; todo &= todo - 1u) {{\n"
            f"       const int l = l0 + __ffs(todo) - 1;\n"
            f"       setup_tile(p, t, (unsigned int)(row * 32 + l), false, false);\n"
            f"       S bb[8]; load_basis(p, t, bb); const uint32_t {basis_decl};\n"
            f"       const uint3 cr = bg_cand_{j}(t, runs_s + l, {basis_names});\n"
            f"       gw[{j}] |= ((cr.x >> t.lane) & 1u) << l;\n"
            f"       pw[{j}] = (pw[{j}] & ~(((cr.y >> t.lane) & 1u) << l)) | (((cr.z >> t.lane) & 1u) << l);\n"
            f"     }}\n"
            f"   }}\n")
    gen.lines, gen.indent, gen.scopes = saved
    live_needs = [(c, dl, mask & ~always) for (c, dl), mask in sorted(need_masks.items())
                  if mask & ~always]
    # a lane can be all ones in an obligation class only if its first four bytes are in it:
    # one table lookup per byte (bit i of obl_tab[b]: byte b is in the i-th class) decides
    # for most tiles that no obligation holds, before any class is computed from the basis
    obl_classes = sorted({c for c, _, _ in live_needs})
    obl_tab = [0] * 256
    if 0 < len(obl_classes) <= 32:
        for i, c in enumerate(obl_classes):
            # a stream that is not a class bounds nothing about the lane's own bytes
            bs = gen.byteset(c) if d.is_cc(c) else full256
            for b in range(256):
                if (bs >> b) & 1:
                    obl_tab[b] |= 1 << i
    else:
        obl_tab = [0xFFFFFFFF] * 256
    obl_lanes = 0
    for _, dl, _ in live_needs:
        obl_lanes |= 1 << dl
        if sl + dl < 32:
            obl_lanes |= 1 << (sl + dl)
    if live_needs:
        gen.open(f"__ballot_sync(FULL, first4_classes(raw, bg_obl_s) != 0u) & 0x{obl_lanes:08x}u")
        if not basis_always:
            gen.emit(basis_block)
    # when one class contains all the others, a lane that is not all ones in it is not all ones
    # in any: test that class at the carry lanes first and skip the rest (the common case)
    guard = None
    if len({c for c, _, _ in live_needs}) > 1 and all(d.is_cc(c) for c, _, _ in live_needs):
        sup = max((c for c, _, _ in live_needs), key=lambda c: (bin(gen.byteset(c)).count("1"), c))
        if all(gen.byteset(c) & ~gen.byteset(sup) == 0 for c, _, _ in live_needs):
            lanes = 0
            for _, dl, _ in live_needs:
                lanes |= 1 << dl
                if sl + dl < 32:
                    lanes |= 1 << (sl + dl)
            guard = sup
            ref = gen.mat(sup)
            gen.emit(f"const uint32_t {pm_classes[sup]} = ones_lanes(t, {gen.pack(ref)});")
            gen.open(f"{pm_classes[sup]} & 0x{lanes:08x}u")
    for c, pm in sorted(pm_classes.items()):
        if c == guard or c not in obl_classes:
            continue
        ref = gen.mat(c)
        gen.emit(f"const uint32_t {pm} = ones_lanes(t, {gen.pack(ref)});")
    for c, dl, mask in live_needs:
        pm = pm_classes[c]
        ors = " ".join(f"runs_s[{32 * w} + l] |= 0x{(mask >> (32 * w)) & 0xFFFFFFFF:08x}u;"
                       for w in range(nw) if (mask >> (32 * w)) & 0xFFFFFFFF)
        gen.emit(f"if (t.lane == 0 && ((({pm} >> {dl}) | ({pm} >> {sl + dl})) & 1u)) {{ {ors} }}")
    if guard is not None:
        gen.close()
    if live_needs:
        gen.close()
    # run masks: kept in the warp's shared words, stored per chunk (flush_runs)
    nonmerged_zero = ""
    if merge:                            # parts OR into the outputs: start every word at zero
        gen.emit(f"if (zin < 0) zero_outputs(p, t, {len(names)});   /* else zeroed per chunk */")
    else:
        # outputs of parts that do not run on a tile are written as zeros, once the chunk's run
        # words are complete
        zs = []
        for ci, outs_k in enumerate(parts):
            cond = " | ".join(f"(runs_s[{32 * w} + l] & 0x{m:08x}u)" for w, m in sorted(part_masks[ci].items())) or "0u"
            zs.append(f"     if (!({cond})) {{ " + " ".join(f"zero_store(p, t, {o});" for o in outs_k) + " }")
        nonmerged_zero = ("   for (int l = l0; l < l0 + CT && row * 32 + l < p.n_tiles; ++l) {\n"
                          "     setup_tile(p, t, (unsigned int)(row * 32 + l), false, false);\n"
                          + "\n".join(zs) + "\n   }\n")
    cls_code = "\n".join(gen.lines)
    log2, keys, info_tab, rec_tab = filt.exact()
    # classify's shared memory: Bloom bitmap, exact table, the warps' run masks.  Programs with
    # many terms (long run masks) get fewer warps per block, then a smaller bitmap.
    bloom_bits = tuning.bloom_bits
    cls_block = max(32, min(1024, tuning.cls_block // 32 * 32))

    hit_cap = 128 * wpt                # Bloom-hit records per warp (BG_HIT_CAP)
    zero_bytes = 4096                  # zeros in shared memory, the bulk zeroing's source

    def cls_words(bits, block):     # up to the warps' hit records (16-byte aligned)
        w = ((1 << bits) // 32 + len(keys) + len(info_tab) + 256
             + (block // 32) * nw * 32 + -(-nw // 4) * 4)
        return -(-w // 4) * 4

    def cls_bytes(bits, block):
        return 4 * cls_words(bits, block) + (block // 32) * 8 * hit_cap + zero_bytes

    while cls_bytes(bloom_bits, cls_block) > 227 * 1024:
        if cls_block > 256:
            cls_block //= 2
        elif bloom_bits > 16:
            bloom_bits -= 1
        else:
            raise NotFusable(f"classify needs {cls_bytes(bloom_bits, cls_block)} bytes of shared memory")
    bloom = filt.bloom(bloom_bits)
    tables = (f"#define BG_EXLOG2 {log2}\n"
              f"static __device__ const __align__(16) uint32_t bg_bloom_g[{len(bloom)}] = {{\n{_hex_array(bloom)}\n}};\n"
              f"static __device__ const __align__(16) uint32_t bg_exkeys[{len(keys)}] = {{\n{_hex_array(keys)}\n}};\n"
              f"static __device__ const __align__(16) uint32_t bg_exinfo[{len(info_tab)}] = {{\n{_hex_array(info_tab)}\n}};\n"
              f"static __device__ const uint32_t bg_exrecs[{len(rec_tab)}] = {{\n{_hex_array(rec_tab)}\n}};\n"
              f"static __device__ const __align__(16) uint32_t bg_obl[256] = {{\n{_hex_array(obl_tab)}\n}};\n"
              f"static __device__ const uint32_t bg_always[{nw}] = {{\n{_hex_array(always_words)}\n}};\n")
    cls_warps = cls_block // 32
    cls_smem = cls_bytes(bloom_bits, cls_block)
    cls_maxreg = max(32, min(255, 65536 // cls_block // 8 * 8))
    cls_kernel = (
        f"//@@BG_PART\n" + ("" if inline else f"//@@BG_UNITREG {cls_maxreg}\n") + f"{tables}"
        f"/* per part: {pmw} (run-mask word, mask) pairs; read by the runtime's work-list kernel */\n"
        f'extern "C" __device__ const uint32_t bg_pmask[{len(pm_table)}] = {{\n{_hex_array(pm_table)}\n}};\n'
        + "".join(cand_funcs) +
        f"/* classify launch: threads per block, bytes of dynamic shared memory (read by the runtime) */\n"
        f'extern "C" __device__ const uint32_t bg_cls_cfg[2] = {{{cls_block}u, {cls_smem}u}};\n'
        f'extern "C" __global__ void __launch_bounds__({cls_block}, 1) {name}_cls(const __grid_constant__ BgParams p) {{\n'
        f"  extern __shared__ __align__(16) uint32_t bg_dyn_s[];\n"
        f"  cls_prologue(p, {len(names)});\n"
        f"  uint32_t *bg_bloom_s = bg_dyn_s;                            /* {len(bloom)} words */\n"
        f"  uint32_t *bg_exkeys_s = bg_dyn_s + {len(bloom)};            /* {len(keys)} words */\n"
        f"  uint32_t *bg_exinfo_s = bg_exkeys_s + {len(keys)};         /* {len(info_tab)} words */\n"
        f"  uint32_t *bg_obl_s = bg_exinfo_s + {len(info_tab)};        /* 256 words */\n"
        f"  uint32_t *bg_runs_s = bg_obl_s + 256;                     /* {cls_warps * nw * 32} words */\n"
        f"  uint32_t *bg_always_s = bg_runs_s + {cls_warps * nw * 32};  /* {nw} words */\n"
        f"  /* the tables, 16 bytes per load with several loads in flight (sizes are multiples of 4 words);\n"
        f"     the exact table's records, read only for a q-gram found in it, stay in global memory */\n"
        f"#pragma unroll 4\n"
        f"  for (int i = threadIdx.x; i < {len(bloom) // 4}; i += blockDim.x)\n"
        f"    reinterpret_cast<uint4 *>(bg_bloom_s)[i] = reinterpret_cast<const uint4 *>(bg_bloom_g)[i];\n"
        f"  for (int i = threadIdx.x; i < {len(info_tab) // 4}; i += blockDim.x)\n"
        f"    reinterpret_cast<uint4 *>(bg_exinfo_s)[i] = reinterpret_cast<const uint4 *>(bg_exinfo)[i];\n"
        f"  for (int i = threadIdx.x; i < 64; i += blockDim.x)\n"
        f"    reinterpret_cast<uint4 *>(bg_obl_s)[i] = reinterpret_cast<const uint4 *>(bg_obl)[i];\n"
        f"  for (int i = threadIdx.x; i < {nw}; i += blockDim.x) bg_always_s[i] = bg_always[i];\n"
        f"  for (int i = threadIdx.x; i < {len(keys) // 4}; i += blockDim.x)\n"
        f"    reinterpret_cast<uint4 *>(bg_exkeys_s)[i] = reinterpret_cast<const uint4 *>(bg_exkeys)[i];\n"
        f"  __syncthreads();\n"
        f"  uint32_t *runs_s = bg_runs_s + (threadIdx.x >> 5) * {nw * 32};\n"
        f"  ClsCtx cx;\n"
        f"  cx.bloom = bg_bloom_s; cx.keys = bg_exkeys_s; cx.info = bg_exinfo_s; cx.recs = bg_exrecs;\n"
        f"  cx.always = bg_always_s; cx.log2 = BG_EXLOG2; cx.runs_s = runs_s; cx.n_hits = 0; cx.row = 0;\n"
        f"  cx.hits_s = reinterpret_cast<uint2 *>(bg_dyn_s + {cls_words(bloom_bits, cls_block)}) + (threadIdx.x >> 5) * BG_HIT_CAP;\n"
        f"  /* {zero_bytes} bytes of zeros, read by the bulk copies that zero the outputs (16-byte aligned) */\n"
        f"  uint32_t *bg_zero_s = bg_dyn_s + {cls_words(bloom_bits, cls_block) + cls_warps * 2 * hit_cap};\n"
        f"  for (int i = threadIdx.x; i < {zero_bytes // 16}; i += blockDim.x)\n"
        f"    reinterpret_cast<uint4 *>(bg_zero_s)[i] = make_uint4(0u, 0u, 0u, 0u);\n"
        f"  asm volatile(\"fence.proxy.async.shared::cta;\" ::: \"memory\"); /* visible to the copy engine */\n"
        f"  __syncthreads();\n"
        f"  const uint32_t zsm = (uint32_t)__cvta_generic_to_shared(bg_zero_s);\n"
        f"  Tile t;\n"
        f"  init(p, t);\n"
        + CLS_CHUNK_OPEN.replace("@ZERO@", (f"zero_chunk_bulk(p, zin, g0, g1, {len(names)}, t.lane, zsm, {zero_bytes}u);"
                                             if tuning.bulk_zero else
                                             f"zero_chunk(p, zin, g0, g1, {len(names)}, t.lane);") if merge else "") +
        f"    if (zin >= 0) setup_tile_in(p, t, (unsigned int)g, zin, zfirst, zn);\n"
        f"    else setup_tile(p, t, (unsigned int)g, false, true);\n"
        f"    uint32_t raw[BG_WPT][8];\n"
        f"    const bool have = pf;\n"
        f"    if (have) {{\n"
        f"#pragma unroll\n"
        f"      for (int j = 0; j < BG_WPT; ++j)\n"
        f"#pragma unroll\n"
        f"        for (int q = 0; q < 8; ++q) raw[j][q] = nraw[j][q];\n"
        f"    }}\n"
        f"    /* the next tile's bytes, loaded while this one is scanned (same input: consecutive) */\n"
        f"    pf = zin >= 0 && p.input_kind == BG_INPUT_BYTES && l + 1 < l0 + CT && g + 1 < p.n_tiles;\n"
        f"    if (pf) {{\n"
        f"#pragma unroll\n"
        f"      for (int j = 0; j < BG_WPT; ++j) load_word_bytes_ahead(p, t, SW, j, nraw[j]);\n"
        f"    }}\n"
        f"    load_scan(p, t, raw, cx, l, have);\n"
        f"    constexpr bool E = true;\n"
        f"{cls_code}\n"
        + CLS_CHUNK_CLOSE.replace("@ROWRUN@", f"p.work + BG_WORK_HEAD + {len(parts)}LL * (1 + rows)")
                         .replace("@CHUNKEND@", "   if (cx.n_hits) resolve_hits(p, cx, t.lane);\n"
                                  + "".join(cand_calls) + nonmerged_zero) +
        f"  if (t.lane == 0) bulk_wait();   /* this warp's zeroing copies are complete */\n"
        f"}}\n")
    warps_per_smsp = -(-(tuning.block // 32) * max(1, tuning.min_blocks) // 4)
    maxreg = max(32, min(255, (16384 // (warps_per_smsp * 32)) // 8 * 8))
    comments = "\n".join(f"/* output {o}: {nm.replace('*/', '* /')} */" for o, nm in enumerate(names))
    src = (
        f"//@@BG_MAXREG {min(maxreg, cls_maxreg) if inline else maxreg}\n"
        f"#define BG_WPT {wpt}\n"
        f"#define BG_HL {gen.hl}\n"
        f"#define BG_TL {gen.tl}\n"
        f"#define BG_NOUT {len(names)}\n"
        f"#define BG_WCOUNT {len(names) if len(names) <= WCOUNT_MAX else 0}\n"
        f"#define BG_LOOKBACK_INLINE {int(tuning.inline_lookback)}\n"
        f"#define BG_LBK {tuning.lookback_width}\n"
        f"#define BG_LB_SPIN {tuning.lookback_spin}\n"
        f"#define BG_NPRE {len(gen.pre)}\n"
        f"#define BG_NRUN {nw}\n"
        f"#define BG_BLOOM_BITS {bloom_bits}\n"
        f"#define BG_QGRAM {filt.q}\n"
        f"#define BG_HIT_CAP {hit_cap}\n"
        f"#define BG_STRIDE {filt.stride}\n"
        f"#define BG_WILD {int(bool(filt.wild_old)) | 2 * int(bool(filt.wild_new))}\n"
        f"#define BG_PREFILTER 1\n"
        f"#define BG_BASIS_FILTER {int(tuning.basis_filter)}\n"
        f'#include "bg_device.cuh"\n'
        f"using namespace bg;\n"
        f"#define VM(j) (E ? t.vm.w[j] : 0xffffffffu)\n"
        f"#define EM(j) (E ? t.em.w[j] : 0xffffffffu)\n"
        f"{comments}\n"
        + "\n".join(funcs) + cls_kernel +
        f"//@@BG_KERNEL\n{decls}\n{fn_tab}"
        f'extern "C" __global__ void __launch_bounds__({tuning.block}, {tuning.min_blocks}) {name}(const __grid_constant__ BgParams p) {{\n'
        f"  __shared__ uint32_t bg_pm_s[{len(pm_table)}];\n"
        f"  for (int i = threadIdx.x; i < {len(pm_table)}; i += blockDim.x) bg_pm_s[i] = bg_pmask[i];\n"
        f"  asm volatile(\"griddepcontrol.wait;\" ::: \"memory\"); /* launched as a programmatic dependent of the row kernel */\n"
        f"  __shared__ uint32_t bg_acc[{warps} * {nacc} * BG_WPT * 32];\n"
        f"  uint32_t *acc = bg_acc + (threadIdx.x >> 5) * ({nacc} * BG_WPT * 32);\n"
        f"  Tile t;\n"
        f"  init(p, t);\n"
        f"  __shared__ unsigned long long bg_cnt_s[{warps} * BG_WCOUNT + 1];\n"
        f"  if (BG_WCOUNT > 0) count_cache_begin(t, bg_cnt_s + (threadIdx.x >> 5) * BG_WCOUNT);\n"
        f"  __shared__ unsigned int bg_pref[{len(parts) + 1}];\n"
        f"  __shared__ unsigned int bg_spent;  /* bit g: the block saw group g's items run out */\n"
        f"  if (threadIdx.x == 0) bg_spent = 0u;\n"
        f"  if (threadIdx.x < 32) {{\n"
        f"    /* group-major, then part-major order (bg_ord): exclusive prefix of the row counts */\n"
        f"    const int per = ({len(parts)} + 31) / 32, lo = threadIdx.x * per;\n"
        f"    unsigned int sum = 0u;\n"
        f"    for (int i = lo; i < lo + per && i < {len(parts)}; ++i) sum += __ldg(p.work + BG_WORK_HEAD + bg_ord[i]);\n"
        f"    unsigned int incl = sum;\n"
        f"    for (int d = 1; d < 32; d <<= 1) {{\n"
        f"      const unsigned int y = __shfl_up_sync(FULL, incl, d);\n"
        f"      if ((int)threadIdx.x >= d) incl += y;\n"
        f"    }}\n"
        f"    unsigned int at = incl - sum;\n"
        f"    for (int i = lo; i < lo + per && i < {len(parts)}; ++i) {{ bg_pref[i] = at; at += __ldg(p.work + BG_WORK_HEAD + bg_ord[i]); }}\n"
        f"    if (threadIdx.x == 31) bg_pref[{len(parts)}] = incl;\n"
        f"  }}\n"
        f"  __syncthreads();\n"
        f"  const long long rows = (p.n_tiles + 31) >> 5;\n"
        f"  /* the warps of an SM start on their group's parts (fewer part bodies per SM in the\n"
        f"     instruction caches) and take other groups' items once their own run out */\n"
        f"  unsigned int smid;\n"
        f"  asm(\"mov.u32 %0, %%smid;\" : \"=r\"(smid));\n"
        f"  int grp = (int)(smid % {ngroups}u), tried = 0;\n"
        f"  /* a warp claims {tuning.exec_claim} consecutive items at once and loads their work-list entries and run\n"
        f"     words together, so that those loads overlap; it then runs them in order (same part:\n"
        f"     rows increasing) */\n"
        f"  for (;;) {{\n"
        f"    const unsigned int gb = bg_pref[bg_gpos[grp]], ge = bg_pref[bg_gpos[grp + 1]];\n"
        f"    unsigned int it0 = 0u;\n"
        f"    if (t.lane == 0)\n"
        f"      it0 = gb < ge && !((*(volatile unsigned int *)&bg_spent >> grp) & 1u) ? gb + atomicAdd(p.work + grp * BG_CLAIM_STRIDE, {tuning.exec_claim}u) : ge;\n"
        f"    it0 = __shfl_sync(FULL, it0, 0);\n"
        f"    if (it0 >= ge) {{\n"
        f"      if (t.lane == 0) atomicOr(&bg_spent, 1u << grp);\n"
        f"      if (++tried >= {ngroups}) break;\n"
        f"      grp = grp + 1 < {ngroups} ? grp + 1 : 0;\n"
        f"      continue;\n"
        f"    }}\n"
        f"    int kq[{tuning.exec_claim}];\n"
        f"    long long g0q[{tuning.exec_claim}];\n"
        f"    uint32_t wantq[{tuning.exec_claim}];\n"
        + "".join(f"    uint32_t rwq{i}[{tuning.exec_claim}];\n" for i in range(pmw)) +
        f"#pragma unroll\n"
        f"    for (int q = 0; q < {tuning.exec_claim}; ++q) {{\n"
        f"      const unsigned int it = it0 + q;\n"
        f"      kq[q] = -1; g0q[q] = 0; wantq[q] = 0u;\n"
        + "".join(f"      rwq{i}[q] = 0u;\n" for i in range(pmw)) +
        f"      if (it < ge) {{\n"
        f"        int j = bg_gpos[grp], hi = bg_gpos[grp + 1];\n"
        f"        while (hi - j > 1) {{ const int m = (j + hi) >> 1; if (bg_pref[m] <= it) j = m; else hi = m; }}\n"
        f"        const int k = bg_ord[j];\n"
        f"        kq[q] = k;\n"
        f"        g0q[q] = (long long)__ldg(p.work + BG_WORK_HEAD + {len(parts)} + (long long)k * rows + (it - bg_pref[j])) * 32;\n"
        f"        const long long g = g0q[q] + t.lane;\n"
        f"        /* each lane loads its tile's run words of the part */\n"
        + "".join(f"        {{ const uint32_t w = bg_pm_s[(k * {pmw} + {i}) * 2], m = bg_pm_s[(k * {pmw} + {i}) * 2 + 1];\n"
                  f"          if (m && g < p.n_tiles) rwq{i}[q] = p.runs[(long long)w * p.n_tiles + g];\n"
                  f"          wantq[q] |= rwq{i}[q] & m; }}\n" for i in range(pmw)) +
        f"      }}\n"
        f"    }}\n"
        f"#pragma unroll\n"
        f"    for (int q = 0; q < {tuning.exec_claim}; ++q) {{\n"
        f"      const int k = kq[q];\n"
        f"      const long long g0 = g0q[q];\n"
        + "".join(f"      const uint32_t rw{i} = rwq{i}[q];\n" for i in range(pmw)) +
        f"      uint32_t sel = __ballot_sync(FULL, wantq[q] != 0u);\n"
        f"      while (sel) {{\n"
        f"        const int l = __ffs(sel) - 1;\n"
        f"        sel &= sel - 1u;\n"
        f"        setup_tile(p, t, (unsigned int)(g0 + l), true, false);\n"
        f"        S b[8];\n"
        f"        load_basis(p, t, b);\n"
        + dispatch +
        f"      }}\n"
        f"    }}\n"
        f"  }}\n"
        f"  flush_counts(p, t);\n"
        f"}}\n")
    return KernelSpec(source=src, name=name, n_outputs=len(names), n_adds=len(gen.adds),
                      halo_lanes=gen.hl, wpt=wpt, block=tuning.block, max_depth_bits=gen.max_dbits,
                      n_nodes=len(d.nodes), output_names=names, tail_lanes=gen.tl,
                      n_pre=len(gen.pre), n_run=nw, merges=merge, n_parts=len(parts),
                      part_outputs=[list(o) for o in parts])
