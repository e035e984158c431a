"""Failure detection without faulting the GPU: a bounded look-back wait that runs out.

The plan is told to make one tile wait on a record no kernel ever writes, with a short wait
limit; the launch must finish, report BG_ERR_TIMEOUT through bg_plan_sync, and leave the context
usable (the next launch without the fault is exact again).
"""

import numpy as np
import pytest
import torch

from bitgen_gb300 import _native as N
from bitgen_gb300.engine import Program, out_layout, pack_bytes
from bitgen_gb300.regex import compile_group
from tests.helpers import oracle_streams, rand_text, first_diff

pytestmark = pytest.mark.gpu


def test_lookback_wait_limit_reports_timeout(cuda):
    g = compile_group(["a[ab]*b", "x.*y"])
    prog = Program([g])
    text = rand_text(200_000, 5, b"abxy")
    inp = pack_bytes([text])
    offs, words, total = out_layout(inp.lengths)
    plan = prog.plan(inp, offs, total)
    out = torch.empty((prog.n_outputs, total), dtype=torch.uint32, device=cuda)
    stream = torch.cuda.current_stream().cuda_stream
    plan.set_wait_limit(20_000_000, debug_wait_tile=3)     # ~10 ms, tile 3 waits forever
    plan.launch(inp.data.data_ptr(), out.data_ptr(), 0, stream)
    with pytest.raises(N.BitgenError) as e:
        plan.sync(stream)
    assert e.value.status == N.BG_ERR_TIMEOUT
    plan.set_wait_limit(0, debug_wait_tile=-1)
    plan.launch(inp.data.data_ptr(), out.data_ptr(), 0, stream)
    plan.sync(stream)
    want = oracle_streams([g], text)[0]
    assert first_diff(out[0, :words[0]].cpu().numpy(), want) is None
