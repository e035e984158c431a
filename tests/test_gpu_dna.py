"""Genomic motif scan: 64 seeded IUPAC motifs (classes such as [AG], N -> [ACGT], gapped forms
with .{lo,hi}) over synthetic DNA text with N runs and a line feed every 80 bytes.

The CPU test pins the emitted programs to the NFA and Python ``re`` on a short slice.  The GPU
tests compare the fused kernel with the C word-parallel oracle, bit for bit, on a ragged 3 MiB
text with per-group and per-regex outputs.
"""

import re

import numpy as np
import pytest
import torch

from bitgen_gb300 import workloads
from bitgen_gb300.engine import Program, pack_bytes
from bitgen_gb300.regex import compile_group
from oracle import cpu
from oracle.nfa_ref import group_match_ends
from oracle.pablo_ref import run_group
from tests.helpers import first_diff


def _workload(n, seed=6):
    ps = workloads.dna_motifs(64, seed=5)
    text = workloads.plant(workloads.dna_text(n, seed=seed), ps.witnesses, 4096, seed + 1)
    return ps, text


def test_dna_programs_match_nfa_and_re():
    ps, text = _workload(6000)
    data = text.tobytes()
    for grp in ps.groups(4):
        g = compile_group(grp)
        got = run_group(g, text)
        assert got == group_match_ends(grp, data)
        want = 0
        for rx in grp:
            pr = re.compile(rx.encode())
            for e in range(len(data)):
                lo = max(0, e + 1 - 64)
                if any(pr.fullmatch(data, s, e + 1) for s in range(lo, e + 1)):
                    want |= 1 << e
        assert got == want
    assert sum(bin(run_group(compile_group(g), text)).count("1") for g in ps.groups(4)) > 0


@pytest.mark.gpu
@pytest.mark.parametrize("per_regex", [False, True])
def test_dna_scan_matches_c_oracle(cuda, per_regex):
    ps, text = _workload((3 << 20) + 4321)
    groups = [compile_group(g) for g in ps.groups(4)]
    prog = Program(groups, per_regex=per_regex)
    assert prog.fused
    res = prog.scan(pack_bytes([text]))
    torch.cuda.synchronize()
    want, wc = cpu.run_groups(groups, text, per_regex=per_regex)
    got = res.streams.cpu().numpy().view(np.uint32)
    W = res.words[0]
    o = res.word_offsets[0]
    assert len(want) == prog.n_outputs == (64 if per_regex else 4)
    for k, w in enumerate(want):
        d = first_diff(got[k, o:o + W], w)
        assert d is None, (k, d)
    assert res.counts[:, 0].cpu().tolist() == wc
    assert sum(wc) > 0
