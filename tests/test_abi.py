"""CPU checks of the C ABI: the library loads, exports every declared entry point, rejects bad
arguments without a device, and NVRTC compiles generated kernels for sm_103a."""

import ctypes as C
import os
import re

import pytest

from bitgen_gb300 import _native as N
from bitgen_gb300.compiler import Tuning, generate_kernel
from bitgen_gb300.regex import compile_group
from bitgen_gb300 import workloads

HEADER = os.path.join(os.path.dirname(os.path.dirname(__file__)), "include", "bitgen_gb300.h")


def declared():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(bg_[a-z0-9_]+)\s*\(", txt)))


def test_exports_every_declared_symbol(native):
    names = declared()
    assert "bg_transpose" in names and "bg_plan_launch" in names
    for n in names:
        assert hasattr(native, n), n
    assert set(names) <= set(N.SIGNATURES), set(names) - set(N.SIGNATURES)


def test_status_strings(native):
    for s in range(9):
        assert N.status_string(s)
    assert N.status_string(N.BG_ERR_TIMEOUT) == "bounded device wait timed out"


def test_bad_arguments_are_reported(native):
    assert native.bg_transpose(None, None, 32, 1, None) == N.BG_ERR_INVALID
    assert native.bg_transpose(C.c_void_p(16), C.c_void_p(16), 31, 1, None) == N.BG_ERR_INVALID
    assert native.bg_transpose(C.c_void_p(17), C.c_void_p(16), 32, 1, None) == N.BG_ERR_ALIGN
    out = C.c_void_p()
    assert native.bg_program_create(None, C.byref(out)) == N.BG_ERR_INVALID
    bad = (N.Instr * 1)(N.Instr(0, 3, 0, 1, -1, 0))  # writes a basis slot
    assert native.bg_interp_create(bad, 1, 12, None, 0, C.byref(out)) == N.BG_ERR_INVALID
    assert native.bg_plan_launch(None, None, None, None, None) == N.BG_ERR_INVALID
    assert native.bg_plan_stats(None, None, 0, None, None) == N.BG_ERR_INVALID
    assert b"bg_plan_stats" in native.bg_last_error()
    assert b"bg_" in native.bg_last_error() or native.bg_last_error()


@pytest.mark.parametrize("wpt,basis_filter", [(1, False), (2, False), (4, False), (1, True),
                                               (2, True)])
def test_generated_kernels_compile_for_sm103a(native, wpt, basis_filter):
    ps = workloads.throughput_patterns(seed=3, n=32)
    groups = [compile_group(g) for g in ps.groups(2)]
    spec = generate_kernel(groups, Tuning(wpt=wpt, basis_filter=basis_filter))
    assert spec.n_parts > 0 and f"#define BG_BASIS_FILTER {int(basis_filter)}" in spec.source
    buf = C.create_string_buffer(1 << 16)
    src = spec.source.encode()
    rc = native.bg_nvrtc_check(src, len(src), b"bg_scan", buf, len(buf))
    assert rc == N.BG_OK, buf.value.decode()


def test_wildcard_filter_kernels_compile_for_sm103a(native):
    """A stride-2 filter with wildcard 4-grams (their exact records read from global memory)."""
    ps = workloads.throughput_patterns(seed=3, n=256)
    groups = [compile_group(g) for g in ps.groups(16)]
    spec = generate_kernel(groups, Tuning(filter_config=(4, 2)))
    assert spec.n_parts > 0 and "#define BG_STRIDE 2" in spec.source
    assert "#define BG_WILD 0" not in spec.source
    assert "bg_cls_cfg[2] = {1024u" in spec.source      # the tables still fit a full block
    buf = C.create_string_buffer(1 << 16)
    src = spec.source.encode()
    rc = native.bg_nvrtc_check(src, len(src), b"bg_scan", buf, len(buf))
    assert rc == N.BG_OK, buf.value.decode()


def test_runner_configuration_flags():
    """init_kernel reads flags from an object with get_config (the reference's config module
    returns None for an unset key; this one raises KeyError) or from a plain dict."""
    from bitgen_gb300.backend import _cfg_flag

    class Cfg:
        def __init__(self, **kw):
            self.kw = kw

        def get_config(self, key):
            return self.kw[key]

    assert _cfg_flag(Cfg(pass_inst_stats_dyn=1), "pass_inst_stats_dyn")
    assert not _cfg_flag(Cfg(pass_inst_stats_dyn=0), "pass_inst_stats_dyn")
    assert not _cfg_flag(Cfg(), "pass_inst_stats_dyn")
    assert _cfg_flag({"pass_inst_stats_dyn": True}, "pass_inst_stats_dyn")
    assert not _cfg_flag({}, "pass_inst_stats_dyn") and not _cfg_flag(None, "pass_inst_stats_dyn")


@pytest.mark.parametrize("n_parts", [0, 3])
def test_dyn_stats_filled_from_scan_counters(monkeypatch, n_parts):
    """run_fn copies the scan's work counters into the dyn_stats tensor init_kernel returned:
    per part (tiles run, rows) for a split-form program, (tiles, 0) for a single kernel.  The
    program is a stand-in here (no device)."""
    from types import SimpleNamespace
    import torch
    import bitgen_gb300.backend as B

    stats = ({"form": "split", "tiles": 10, "tiles_run": [1, 0, 7], "rows": [1, 0, 2],
              "part_outputs": [[0], [1], [1]]} if n_parts else {"form": "single-kernel", "tiles": 10})

    class Prog:
        fused = True
        spec = SimpleNamespace(n_parts=n_parts)

        def __init__(self, groups, tuning=None):
            pass

        def scan(self, inp, **kw):
            assert kw["stats"] and kw["out_stride"] == 4
            return SimpleNamespace(stats=stats)

        def close(self):
            pass

    monkeypatch.setattr(B, "Program", Prog)
    monkeypatch.setattr(B, "basis_input", lambda basis: None)
    basis = torch.zeros((1, 1, 8, 4), dtype=torch.uint32)
    result, tmp, handle, run_fn, dyn = B.init_kernel(2, None, basis, {"pass_inst_stats_dyn": 1},
                                                     groups=[object(), object()])
    assert tuple(result.shape) == (1, 1, 2, 4) and tmp is None
    assert tuple(dyn.shape) == (1, 1, max(1, n_parts), 2) and int(dyn.sum()) == 0
    run_fn(basis)
    want = [[1, 1], [0, 0], [7, 2]] if n_parts else [[10, 0]]
    assert dyn[0, 0].tolist() == want
    handle.free()


C_HOST = r"""
#include "bitgen_gb300.h"
#include <stdio.h>
#include <string.h>
int main(void) {
  char log[8192];
  const char *src = "extern \"C\" __global__ void k(unsigned int *x) { x[threadIdx.x] = 1u; }";
  int rc = bg_nvrtc_check(src, strlen(src), "k", log, sizeof log);
  if (rc != BG_OK) { printf("nvrtc %d %s\n", rc, log); return 1; }
  if (bg_plan_stats(NULL, NULL, 0, NULL, NULL) != BG_ERR_INVALID) return 2;
  if (strcmp(bg_status_string(BG_ERR_TIMEOUT), "bounded device wait timed out") != 0) return 3;
  if (bg_transpose(NULL, NULL, 32, 1, NULL) != BG_ERR_INVALID) return 4;
  if (bg_plan_launch(NULL, NULL, NULL, NULL, NULL) != BG_ERR_INVALID) return 5;
  puts("ok");
  return 0;
}
"""


def test_c_host_builds_and_calls_the_abi(native, tmp_path):
    """A plain C99 host includes include/bitgen_gb300.h, links the library and calls the entry
    points that need no device (compile-only NVRTC check, argument checks, status strings)."""
    import shutil
    import subprocess
    cc = shutil.which("gcc")
    if cc is None:
        pytest.skip("no host C compiler")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    libdir = os.path.join(root, "bitgen_gb300")
    src = tmp_path / "host.c"
    src.write_text(C_HOST)
    exe = tmp_path / "host"
    subprocess.run([cc, "-std=c99", "-Wall", "-Werror", f"-I{os.path.join(root, 'include')}", str(src),
                    f"-L{libdir}", "-lbitgen_gb300", f"-Wl,-rpath,{libdir}", "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0 and out.stdout.strip() == "ok", (out.returncode, out.stdout, out.stderr)


def test_random_regex_programs_compile_in_both_forms(native):
    """Seeded random regex groups (every emitter construct) generate kernels that NVRTC
    compiles for sm_103a, in the split form and the single-kernel form with and without
    zero-block skipping."""
    import random
    from bitgen_gb300.compiler import NotFusable
    from bitgen_gb300.regex import UnsupportedRegex, _matches_empty, parse_regex
    from tests.test_oracle import _fuzz_regex
    rnd = random.Random(21)
    compiled = 0
    for _ in range(4):
        rs = []
        while len(rs) < 6:
            r = "qz" + _fuzz_regex(rnd, 3) + "k"
            try:
                if not _matches_empty(parse_regex(r)):
                    compile_group([r])
                    rs.append(r)
            except UnsupportedRegex:
                pass
        groups = [compile_group(rs[i::2]) for i in range(2)]
        for t in (Tuning(prefilter=False), Tuning(wpt=1, prefilter_limit=1.0),
                  Tuning(prefilter=False, wpt=2, skip_interval=1)):
            try:
                spec = generate_kernel(groups, t, per_regex=True)
            except NotFusable:
                continue        # programs that keep a while loop run on the whole-stream executor
            buf = C.create_string_buffer(1 << 16)
            src = spec.source.encode()
            rc = native.bg_nvrtc_check(src, len(src), b"bg_scan", buf, len(buf))
            assert rc == N.BG_OK, (rs, buf.value.decode()[:2000])
            compiled += 1
    assert compiled >= 6
