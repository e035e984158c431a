"""CPU: pushing Advances down to the character classes (compiler.push_advances) keeps every
output stream, and the single-kernel code it leads to shifts each class once per distance."""

import numpy as np
import pytest

from bitgen_gb300 import workloads
from bitgen_gb300.compiler import (Tuning, build_dag, generate_kernel, interleave_chains,
                                   push_advances)
from bitgen_gb300.regex import compile_group
from oracle.pablo_ref import basis_ints, matchstar, scanthru


def _eval(dag, outs, data: np.ndarray):
    """Every output of the DAG over `data`, as Python big-int streams (oracle semantics)."""
    n = data.size
    mask = (1 << n) - 1
    basis = basis_ints(data)
    val = {}
    for nd in dag.nodes:
        x = [val[a] for a in nd.args]
        op = nd.op
        if op == "basis":
            r = basis[nd.basis]
        elif op == "zero":
            r = 0
        elif op == "ones":
            r = mask
        elif op == "and":
            r = x[0] & x[1]
        elif op == "or":
            r = x[0] | x[1]
        elif op == "xor":
            r = x[0] ^ x[1]
        elif op == "not":
            r = ~x[0] & mask
        elif op == "sel":
            r = (x[0] & x[1]) | (~x[0] & x[2] & mask)
        elif op == "advance":
            r = (x[0] << nd.shift) & mask
        elif op == "lookahead":
            r = x[0] >> nd.shift
        elif op == "matchstar":
            r = matchstar(x[0], x[1], mask)
        elif op == "scanthru":
            r = scanthru(x[0], x[1], mask)
        else:
            raise AssertionError(op)
        val[nd.id] = r & mask
    return [val[o] for o in outs]


def _cases():
    dna = workloads.dna_motifs(64, seed=5)
    yield "dna", [compile_group(g) for g in dna.groups(4)], \
        workloads.plant(workloads.dna_text(20000, seed=3), dna.witnesses, 400, 4)
    thr = workloads.throughput_patterns(seed=91, n=48)
    yield "throughput", [compile_group(g) for g in thr.groups(4)], \
        workloads.plant(workloads.printable_text(20000, 5), thr.witnesses, 300, 6)
    small, text = workloads.small_workload()
    yield "small", [compile_group(g) for g in small.groups(4)], text


@pytest.mark.parametrize("per_regex", [False, True])
@pytest.mark.parametrize("label,groups,text", list(_cases()), ids=lambda x: x if isinstance(x, str) else "")
def test_pushed_outputs_equal(label, groups, text, per_regex):
    dag, outs, _ = build_dag(groups, per_regex=per_regex)
    want = _eval(dag, outs, text)
    new = push_advances(dag, outs)
    assert _eval(dag, new, text) == want
    assert any(want)
    for batch in (1, 5, 64):
        for pairs in (False, True):
            inter, epochs = interleave_chains(dag, new, batch, pairs)
            assert _eval(dag, inter, text) == want, (batch, pairs)
            assert all(dag.nodes[v].op == "and" for v in epochs)


def test_pushed_dag_shifts_classes_not_markers():
    """On the DNA motifs the rewrite leaves fewer than half the Advances, most of them on the
    16 character classes, and the generated single-kernel code shares the words it reads."""
    dna = workloads.dna_motifs(64, seed=5)
    groups = [compile_group(g) for g in dna.groups(4)]
    dag, outs, _ = build_dag(groups)
    n0 = len(dag.nodes)
    live0, stack = set(), list(outs)
    while stack:
        v = stack.pop()
        if v not in live0:
            live0.add(v)
            stack.extend(dag.nodes[v].args)
    new = push_advances(dag, outs)
    live, stack = set(), list(new)
    while stack:
        v = stack.pop()
        if v not in live:
            live.add(v)
            stack.extend(dag.nodes[v].args)
    adv = [dag.nodes[v] for v in live if dag.nodes[v].op == "advance"]
    before = sum(1 for nd in dag.nodes[:n0] if nd.op == "advance" and nd.id in live0)
    on_class = [a for a in adv if dag.is_cc(a.args[0])]
    # what stays on markers: nodes with several users (the gaps' repetitions, shared prefixes)
    assert len(adv) * 2 < before and len(on_class) * 2 > len(adv)
    assert len({a.args[0] for a in on_class}) <= 16
    spec = generate_kernel(groups, Tuning())
    assert spec.n_parts == 0 and "sr" in spec.source
    off = generate_kernel(groups, Tuning(push_advances=False))
    assert off.source.count("__funnelshift_r") > spec.source.count("__funnelshift_r") or \
        off.source.count("__shfl_up_sync") > spec.source.count("__shfl_up_sync")


def test_cluster_chains_batches_share_classes():
    """Batches are at most `batch` chains, cover every chain once, and a batch formed around
    shared shifted classes needs fewer distinct classes than chains taken in id order."""
    from bitgen_gb300.compiler import _cluster_chains
    leaves = {
        1: [(10, 0), (11, 1)], 2: [(20, 0), (21, 1)], 3: [(10, 0), (11, 1), (12, 2)],
        4: [(20, 0), (21, 1), (22, 2)], 5: [(10, 0)], 6: [(20, 0)],
    }
    members = sorted(leaves)
    groups = _cluster_chains(members, leaves, 3)
    assert sorted(x for g in groups for x in g) == members
    assert all(len(g) <= 3 for g in groups)
    distinct = sum(len({lf for r in g for lf in leaves[r]}) for g in groups)
    in_order = sum(len({lf for r in members[i:i + 3] for lf in leaves[r]}) for i in range(0, 6, 3))
    assert distinct < in_order
    # few chains: one batch, in order
    assert _cluster_chains([3, 1], leaves, 8) == [[3, 1]]


def test_guard_regions_never_read_a_later_block(monkeypatch):
    """A part whose zero-skip regions would open a guard block that reads a node declared for
    a later block (still zero there) is generated as one unguarded region; the programs of the
    benchmark workloads keep their guards."""
    import bitgen_gb300.compiler as C
    used = []
    orig = C._Gen._part

    def spy(self, terms, outer_regs, skip):
        r = orig(self, terms, outer_regs, skip)
        used.append(skip)
        return r

    monkeypatch.setattr(C._Gen, "_part", spy)
    regexes = ["q(rs)*t", "(ab)+c", "x(abc)*y", "(a[0-9]){2,}z", "(ab|cd)*e", "k(xy)*",
               "(?i)(gh)+i", "m(n(op){2})*w"]
    stars = [compile_group(regexes[i::2]) for i in range(2)]
    generate_kernel(stars, Tuning(prefilter=False), per_regex=True)
    assert used == [False]
    used.clear()
    small, _ = workloads.small_workload()
    thr = workloads.throughput_patterns(seed=3, n=64)
    for gs in ([compile_group(g) for g in small.groups(4)], [compile_group(g) for g in thr.groups(4)]):
        generate_kernel(gs, Tuning(prefilter=False))
    assert used and all(used)
