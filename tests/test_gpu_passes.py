"""GPU: programs as BitGen's pass pipeline leaves them run on the engine.

Each instruction list of ``tests/golden/passes.json`` (the reference's ``run_passes`` output
under short_circuit 0/1 and graph_break -1/0/1, see ``tests/test_passes_ir.py``) is converted by
``refir.group_from_ir`` and scanned on the GPU: the fused kernel where its loops are MatchStar
loops, the whole-stream executor otherwise.  Streams must equal the oracle's."""

import json
import os

import numpy as np
import pytest
import torch

from bitgen_gb300 import refir, workloads
from bitgen_gb300.engine import Program, bytes_input
from tests.helpers import first_diff, oracle_streams

pytestmark = pytest.mark.gpu
CASES = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "passes.json")))


@pytest.mark.parametrize("case", sorted(CASES))
def test_pass_output_runs_on_the_engine(cuda, case):
    c = CASES[case]
    group = refir.group_from_ir(c["ir"])
    if c["regexes"]:
        wits = [r.encode() for r in c["regexes"] if r.isalnum()] or [b"x"]
        text = workloads.plant(workloads.printable_text(200_000, 5), wits, 700, 6)
    else:
        rng = np.random.default_rng(5)
        alpha = np.frombuffer(b"<>/=\"' abcxyz\n?!-[]&;", np.uint8)
        text = alpha[rng.integers(0, alpha.size, 50_000)]
    prog = Program([group])
    res = prog.scan(bytes_input(torch.from_numpy(text).to(cuda)))
    got = res.streams[0, :(text.size + 31) // 32].cpu().numpy().view(np.uint32)
    want = oracle_streams([group], text)[0]
    assert first_diff(got, want) is None, (case, prog.fused, first_diff(got, want))
    assert int(res.counts[0, 0]) == int(np.unpackbits(want.view(np.uint8)).sum())
    prog.close()
