"""Build the engine's native library ``libbitgen_gb300.so`` in-tree with nvcc (sm_103a).

The library holds the C ABI (``include/bitgen_gb300.h``), the stand-alone transpose kernel, the
whole-stream executor and the NVRTC driver; the device headers the generated kernels include
are embedded as strings so NVRTC needs nothing from disk at run time.
"""

from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libbitgen_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
EMBED = [("bg_embedded_device_cuh", "bg_device.cuh"),
         ("bg_embedded_params_h", "bg_params.h"),
         ("bg_embedded_transpose_cuh", "bg_transpose.cuh")]
SOURCES = ["bg_runtime.cu", "bg_interp.cu"]


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _cuda_home(nvcc: str) -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def _write_embed() -> str:
    os.makedirs(BUILD, exist_ok=True)
    out = os.path.join(BUILD, "bg_embed.cpp")
    parts = ['/* generated by bitgen_gb300/build.py: device headers for NVRTC */\n']
    for sym, fname in EMBED:
        with open(os.path.join(CSRC, fname)) as f:
            txt = f.read()
        delim = "BGEMBED"
        assert f"){delim}\"" not in txt
        parts.append(f'extern "C" {{\nconst char *{sym} = R"{delim}({txt}){delim}";\n}}\n')
    data = "".join(parts)
    if not os.path.exists(out) or open(out).read() != data:
        with open(out, "w") as f:
            f.write(data)
    return out


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    nvcc = _nvcc()
    home = _cuda_home(nvcc)
    embed = _write_embed()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(os.path.dirname(PKG), "include", "bitgen_gb300.h"))
    objs = []
    jobs = []
    for src in SOURCES + [embed]:
        path = src if os.path.isabs(src) else os.path.join(CSRC, src)
        obj = os.path.join(BUILD, os.path.basename(path) + ".o")
        objs.append(obj)
        if force or _stale(obj, [path] + headers + [__file__]):
            cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                   "-c", path, "-o", obj]
            jobs.append(cmd)

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return r.stderr

    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        for msg in ex.map(run, jobs):
            if verbose and msg:
                print(msg)
    if force or jobs or _stale(LIB, objs):
        libdir = os.path.join(home, "lib64")
        tmp = LIB + ".tmp"
        cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, f"-L{libdir}", "-lnvrtc", "-lnvJitLink",
               "-Xlinker", f"-rpath={libdir}"]
        run(cmd)
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
