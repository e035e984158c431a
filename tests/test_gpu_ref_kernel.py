"""GPU: this engine's match streams equal those of the reference's own generated GPU kernel.

``oracle/ref_gpu.py`` lowers the DNA motif groups through BitGen's passes and ``CudaGenerator``
(``bitgen/codegen/gen_cuda.py:395-497``) with ``--pass-cc-advanced=0`` (outputs at their own
positions) into ``oracle/_ref``; the kernel is compiled for this GPU and launched as
``cuda_kernel.py:411-427`` does (grid = (groups, inputs)).  Skipped where that file was not
generated (it is made where the reference tree is)."""

import numpy as np
import pytest
import torch

from bitgen_gb300 import workloads
from bitgen_gb300.backend import byte_stream_transpose
from bitgen_gb300.engine import Program, bytes_input, pack_bytes
from bitgen_gb300.regex import compile_group
from oracle import ref_gpu

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dna(cuda):
    if not ref_gpu.available(ref_gpu.DNA):
        pytest.skip("the reference's generated DNA kernel was not generated")
    ps = workloads.dna_motifs(64, seed=5)
    groups = ps.groups(4)
    prog = Program([compile_group(g) for g in groups])
    yield ps, groups, prog, ref_gpu.RefKernel(ref_gpu.DNA, groups)
    prog.close()


def _reference(k, text: torch.Tensor, inputs: int):
    words = text.numel() // 32 // inputs
    flat, basis = k.basis_buffer(inputs, words, text.device)
    byte_stream_transpose(text[:inputs * words * 32].view(1, inputs, words * 32), basis)
    res = torch.zeros((inputs, k.groups, words), dtype=torch.uint32, device=text.device)
    k.launch(flat, inputs, words, res, torch.cuda.current_stream(text.device))
    torch.cuda.synchronize()
    return res, words


@pytest.mark.parametrize("n_bytes", [32 * 1000, 1 << 20, 3 * (1 << 20) + 4096])
def test_streams_equal_the_reference_kernel(dna, cuda, n_bytes):
    """One input of DNA text with planted motifs: every group's stream bit for bit."""
    ps, groups, prog, k = dna
    text = torch.from_numpy(workloads.plant(workloads.dna_text(n_bytes, seed=11), ps.witnesses,
                                            2048, 12)).to(cuda)
    res, words = _reference(k, text, 1)
    r = prog.scan(bytes_input(text))
    got = r.streams[:, :words]
    assert int(got.count_nonzero()) > 0
    assert torch.equal(res[0], got)


def test_multi_input_counts_equal(dna, cuda):
    """Twelve inputs on the grid's second axis (multi_input): per-input streams equal the
    engine's batch of the same twelve inputs."""
    ps, groups, prog, k = dna
    n = 12 * 32 * 3000
    text = torch.from_numpy(workloads.plant(workloads.dna_text(n, seed=13), ps.witnesses, 200,
                                            14)).to(cuda)
    res, words = _reference(k, text, 12)
    r = prog.scan(pack_bytes(list(text.view(12, words * 32)), device=cuda))
    for i in range(12):
        o = r.word_offsets[i]
        assert r.words[i] == words
        assert torch.equal(res[i], r.streams[:, o:o + words]), i
