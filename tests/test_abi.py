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


@pytest.mark.parametrize("wpt", [1, 2, 4])
def test_generated_kernels_compile_for_sm103a(native, wpt):
    ps = workloads.throughput_patterns(seed=3, n=32)
    groups = [compile_group(g) for g in ps.groups(2)]
    spec = generate_kernel(groups, Tuning(wpt=wpt))
    buf = C.create_string_buffer(1 << 16)
    src = spec.source.encode()
    rc = native.bg_nvrtc_check(src, len(src), b"bg_scan", buf, len(buf))
    assert rc == N.BG_OK, buf.value.decode()
