"""CPU: the byte <-> basis-plane word transposes of `bg_transpose.cuh`, compiled for the host with
a plain-C++ `__byte_perm` (result byte n = byte `(s >> 4n) & 7` of the pair y:x; every selector
the header uses has nibbles below 8).  `transpose32` must give the reference layout (plane b bit
31-j = bit 7-b of byte j, `bitstream.py:228-258`) and `untranspose32` must invert it."""

import os
import shutil
import subprocess

import pytest

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                      "bitgen_gb300", "csrc", "bg_transpose.cuh")

SRC = r"""
#include <cstdint>
#include <cstdio>
#include <random>
#define __device__
#define __forceinline__ inline
static inline uint32_t __byte_perm(uint32_t x, uint32_t y, uint32_t s) {
  const uint64_t v = (uint64_t)x | ((uint64_t)y << 32);
  uint32_t r = 0;
  for (int n = 0; n < 4; ++n) r |= (uint32_t)((v >> (8 * ((s >> (4 * n)) & 7))) & 0xff) << (8 * n);
  return r;
}
#include HEADER_PATH
int main() {
  std::mt19937 g(7);
  for (int it = 0; it < 200000; ++it) {
    uint32_t u[8], o[8], v[8];
    for (int k = 0; k < 8; ++k) u[k] = it < 256 ? 0x01010101u * (uint32_t)it : (uint32_t)g();
    bg::transpose32(u, o);
    for (int j = 0; j < 32; ++j) {
      const uint32_t byte = (u[j >> 2] >> (8 * (j & 3))) & 0xffu;
      for (int b = 0; b < 8; ++b)
        if (((o[b] >> (31 - j)) & 1u) != ((byte >> (7 - b)) & 1u)) {
          printf("layout it=%d byte=%d plane=%d\n", it, j, b);
          return 1;
        }
    }
    bg::untranspose32(o, v);
    for (int k = 0; k < 8; ++k)
      if (v[k] != u[k]) {
        printf("inverse it=%d word=%d\n", it, k);
        return 1;
      }
  }
  puts("ok");
  return 0;
}
"""


def test_transpose_and_inverse_on_host(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    src = tmp_path / "t.cpp"
    src.write_text(SRC)
    exe = tmp_path / "t"
    subprocess.run([cxx, "-O2", f'-DHEADER_PATH="{HEADER}"', "-o", str(exe), str(src)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0 and out.stdout.strip() == "ok", out.stdout + out.stderr
