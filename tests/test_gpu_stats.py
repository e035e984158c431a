"""GPU: the work counters through the reference-facing hook.  With ``pass_inst_stats_dyn`` set,
``init_kernel`` returns a ``dyn_stats`` tensor that every ``run_fn`` refreshes, and the
reference runner's reductions over it work (``from_icgrep.py:619-640``)."""

import os

import numpy as np
import pytest
import torch

from bitgen_gb300.backend import byte_stream_transpose, init_kernel
from bitgen_gb300.grouping import group_regex_in_list
from bitgen_gb300.regex import compile_group
from bitgen_gb300 import workloads

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


class _Config:
    """A runner configuration with get_config, as the reference's config module offers."""

    def __init__(self, **flags):
        self.flags = flags

    def get_config(self, key):
        return self.flags.get(key)


def _basis(data: np.ndarray, dev):
    """bitgen/bitstream.py:166-225: pad to 32, uint8 [1, 1, Npad] -> uint32 [1, 1, 8, W]."""
    npad = -(-data.size // 32) * 32
    bytestream = torch.zeros((1, 1, npad), dtype=torch.uint8, device=dev)
    bytestream[0, 0, :data.size] = torch.from_numpy(data.copy())
    basis = torch.zeros((1, 1, 8, npad // 32), dtype=torch.uint32, device=dev)
    byte_stream_transpose(bytestream, basis)
    return bytestream, basis, npad


def _reference_reductions(dyn: torch.Tensor):
    """What the reference runner computes from dyn_stats (from_icgrep.py:620-636)."""
    iter_num, dyn_offset_num = dyn[..., :1], dyn[..., 1:]
    return (iter_num.sum().item(), dyn_offset_num.sum().item(),
            dyn_offset_num.to(torch.float32).max().item(),
            dyn_offset_num.to(torch.float32).std().item() if dyn_offset_num.numel() > 1 else 0.0,
            dyn.sum().item())


def test_dyn_stats_single_kernel_program(cuda):
    """The reference's quick-start program compiles to the single-kernel form: one row of
    counters, the tiles of the launch."""
    kat = np.load(os.path.join(GOLDEN, "readme_kat.npz"))
    rx = [str(r) for r in kat["regexes"]]
    groups = [compile_group(g) for g in group_regex_in_list(rx, int(kat["n_groups"]))]
    bytestream, basis, npad = _basis(kat["input"], cuda)
    result, tmp, handle, run_fn, dyn = init_kernel(len(groups), bytestream, basis,
                                                   _Config(pass_inst_stats_dyn=True), groups=groups)
    prog = handle.program
    assert prog.fused and prog.spec.n_parts == 0
    assert tuple(dyn.shape) == (1, 1, 1, 2) and int(dyn.sum()) == 0
    run_fn(basis)
    torch.cuda.synchronize()
    assert int(np.unpackbits(result.cpu().numpy().view(np.uint8)).sum()) == 16
    tiles = prog.tiles_for([npad])
    assert dyn[0, 0, 0].tolist() == [tiles, 0]
    assert _reference_reductions(dyn)[0] == tiles
    handle.free()
    assert init_kernel(len(groups), bytestream, basis, _Config(), groups=groups)[4] is None


@pytest.mark.parametrize("basis_filter", [True, False])
def test_dyn_stats_split_program(cuda, basis_filter):
    """64 regexes over printable text compile to the split form: per part the tiles it ran on
    and the rows of its work list, the same on every run.  The hook scans basis planes: by
    default the classify pass rebuilds their bytes and runs the q-gram filter, so parts run on
    few tiles; with Tuning(basis_filter=False) every part runs on every tile and lists every
    row.  The streams equal the oracle's either way."""
    from bitgen_gb300.compiler import Tuning
    from oracle.pablo_ref import int_to_words, run_group
    ps = workloads.throughput_patterns(seed=91, n=64)
    groups = [compile_group(g) for g in ps.groups(4)]
    data = workloads.plant(workloads.printable_text(200_000, 94), ps.witnesses, 4096, 95)
    bytestream, basis, npad = _basis(data, cuda)
    result, tmp, handle, run_fn, dyn = init_kernel(len(groups), bytestream, basis,
                                                   {"pass_inst_stats_dyn": True}, groups=groups,
                                                   tuning=Tuning(basis_filter=basis_filter))
    prog = handle.program
    assert prog.fused and prog.spec.n_parts > 0
    assert tuple(dyn.shape) == (1, 1, prog.spec.n_parts, 2)
    run_fn(basis)
    torch.cuda.synchronize()
    padded = np.concatenate([data, np.zeros(npad - data.size, np.uint8)])
    for g, grp in enumerate(groups):
        want = int_to_words(run_group(grp, padded), npad // 32)
        assert np.array_equal(result[0, 0, g].cpu().numpy().view(np.uint32), want), g
    tiles = prog.tiles_for([npad])
    runs, rows = dyn[0, 0, :, 0].tolist(), dyn[0, 0, :, 1].tolist()
    if basis_filter:
        assert all(0 <= r <= tiles for r in runs) and sum(runs) < prog.spec.n_parts * tiles // 4
        assert all(0 <= r <= -(-tiles // 32) for r in rows)
    else:
        assert runs == [tiles] * prog.spec.n_parts
        assert rows == [-(-tiles // 32)] * prog.spec.n_parts
    red = _reference_reductions(dyn)
    assert red[0] == sum(runs) and red[1] == sum(rows) and red[2] >= 1.0
    first = dyn.clone()
    run_fn(basis)
    torch.cuda.synchronize()
    assert torch.equal(dyn, first)
    handle.free()
