"""Benchmark: input GB/s of the fused bitstream scan on the 256-regex throughput workload.

Workload (one step = one scan of the whole input): 256 seeded synthetic regexes of the
benchmark grammar (4-12-byte literals mixed with [a-z0-9] classes, {2,5} repeats, a .* gap, a
2-way alternation), 16 groups of 16, over 1 MiB of printable ASCII with planted matches, tiled
to 256 MiB.  Each step writes the 16 per-group match streams (the reference's result shape) and
the per-group match counts.  The input (256 MiB) is larger than L2 (129 MB), so no flush is
needed between steps.  The CPU evaluator scans the same 256 MiB once; the streams and counts of
the timed launches must equal its own.

Further legs on the same line: ``positions_only`` and ``basis_hook`` (the same scan with
positions instead of streams, and through the reference's run_fn(basis) hook), ``batched``
(4096 small inputs, one graph launch vs one launch per input, with an autotune report),
``transpose``, ``dna`` (64 IUPAC motifs over 1 GiB of DNA text, its own CPU check, and the
reference's generated kernel timed beside it) and ``served`` (Poisson request arrivals over
three resident pattern sets, p50/p99 latency).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

``--impl reference`` times the CPU evaluator (``oracle/bg_cpu.c``, all host threads) on the same
workload, one scan of the 256 MiB input per step: the reference's CPU comparison point, icgrep,
is not part of the reference tree, and its GPU path cannot run these programs (its parser
rejects MatchStar; the while-loop form needs whole-stream loop tests its kernel does per tile).
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "input GB/s @256 regexes (bit-exact)"
UNIT = "GB/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--bytes", type=int, default=256 << 20, help="input bytes per GPU")
    ap.add_argument("--regexes", type=int, default=256)
    ap.add_argument("--groups", type=int, default=16)
    ap.add_argument("--wpt", type=int, default=0, help="words per lane (0 = autotuned default)")
    ap.add_argument("--cpu-sample", type=int, default=0,
                    help="bytes of the CPU baseline sample (0 = the whole input, a few seconds)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-modes", action="store_true", help="skip the batched / transpose / DNA / served legs")
    ap.add_argument("--served-requests", type=int, default=20000)
    ap.add_argument("--dna-bytes", type=int, default=1 << 30, help="DNA text of the dna leg")
    ap.add_argument("--no-ref-gpu", action="store_true",
                    help="skip the reference's generated kernel in the dna leg (profiling runs)")
    ap.add_argument("--served-only", action="store_true",
                    help="run only the served leg and print its JSON")
    ap.add_argument("--dna-only", action="store_true",
                    help="run only the dna leg and print its JSON (profiling the DNA kernel)")
    return ap.parse_args()


def workload(args):
    import numpy as np
    from bitgen_gb300 import workloads
    ps, base, reps = workloads.throughput_workload(total_bytes=args.bytes, n_regex=args.regexes)
    groups = ps.groups(args.groups)
    return ps, groups, base, reps


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, index: int):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                       "-i", str(index), "-lms", "200"], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        time.sleep(0.3)
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.seek(0)
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f.read().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = max(mx, float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.f.name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_baseline(groups, base, sample_bytes):
    """C evaluator on the host over a bounded sample (the first `sample_bytes` of `base` tiled),
    on every host core: one group per thread, or, for programs of bounded reach (no additions
    or loops), one byte range per thread.  Its streams and counts are the bit-exact check of
    the GPU run.  Returns (baseline record, streams, counts)."""
    import numpy as np
    from oracle import cpu
    from bitgen_gb300.engine import lower_interp
    from bitgen_gb300.regex import compile_group

    gs = [compile_group(g) if isinstance(g, list) else g for g in groups]
    reps = -(-sample_bytes // base.size)
    data = np.tile(base, reps)[:sample_bytes] if reps > 1 else base[:sample_bytes]
    cores = os.cpu_count() or 1
    split = all(cpu.reach(lower_interp([g])[0]) is not None for g in gs) and len(gs) < cores
    threads = cores if split else min(cores, len(gs))
    cpu.run_groups(gs, data[:1 << 16], threads=threads)  # warm
    t0 = time.perf_counter()
    streams, counts = cpu.run_groups(gs, data, threads=threads, split=split)
    dt = time.perf_counter() - t0
    how = (f"one byte range per thread ({threads} ranges)" if split else "one group per thread")
    return {"value": round(sample_bytes / dt / 1e9, 6), "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{sample_bytes} bytes of the same input, all {len(gs)} groups, {how} "
                      f"(C word-parallel evaluator, oracle/bg_cpu.c), {dt:.2f} s"}, streams, counts


def streams_equal(out, cpu_streams, words: int) -> bool:
    """Every output stream of a GPU launch (device uint32 [n_out, >= words]) equals the CPU
    evaluator's over all `words` words."""
    import numpy as np
    got = out[:, :words].cpu().numpy().view(np.uint32)
    return len(cpu_streams) == got.shape[0] and all(
        np.array_equal(got[k], np.asarray(cpu_streams[k][:words], dtype=np.uint32))
        for k in range(got.shape[0]))


def batched_leg(prog, gs, ps, dev):
    """4096 inputs, log-normal lengths (median 8 KiB, sigma 1, 200 B - 64 KiB): one persistent
    CUDA-graph launch vs one launch per input, same GPU, outputs compared bit for bit.  The
    program's tuning is chosen by the autotuner on a sample of 512 of the inputs."""
    import numpy as np
    import torch
    from dataclasses import asdict
    from bitgen_gb300 import workloads
    from bitgen_gb300.autotune import autotune
    from bitgen_gb300.batched import BatchScanner, PerInputScanner
    from bitgen_gb300.compiler import Tuning
    from bitgen_gb300.engine import Program, pack_bytes

    lens = workloads.batched_lengths(4096, seed=7)
    items = workloads.batched_inputs(lens, 7, ps.witnesses)
    total = int(sum(lens))
    space = [Tuning(), Tuning(part_cap=1), Tuning(part_cap=4, exec_groups=8)]
    t0 = time.perf_counter()
    best, report = autotune(gs, pack_bytes(items[:512], device=dev), space=space, use_cache=False)
    tune_s = time.perf_counter() - t0
    default = asdict(Tuning())

    def diff(t):
        return {k: v for k, v in t.items() if default.get(k) != v}
    if asdict(best) != default:
        prog = Program(gs, tuning=best)
    b = BatchScanner(prog, items, device=dev, graph=True)
    p = PerInputScanner(prog, items, device=dev)
    for _ in range(2):
        b.run(); b.sync(); p.run(); p.sync()

    def timed(sc, reps):
        s = sc.stream
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        for _ in range(reps):
            sc.run()
        e1.record(s)
        sc.sync()
        return e0.elapsed_time(e1) / reps

    tb = timed(b, 10)
    tp = timed(p, 3)
    # the inputs' words (the alignment gaps between them are written by neither form)
    idx = torch.from_numpy(np.concatenate([np.arange(o, o + w) for o, w in zip(b.offs, b.words)])
                           ).to(dev)
    exact = bool(torch.equal(b.counts, p.counts) and
                 torch.equal(b.out.index_select(1, idx), p.out.index_select(1, idx)))
    return {"inputs": len(items), "bytes": total, "graph": True,
            "batched_GBps": round(total / tb / 1e6, 3), "plain_GBps": round(total / tp / 1e6, 3),
            "batched_ms": round(tb, 4), "plain_ms": round(tp, 4), "speedup": round(tp / tb, 2),
            "plain_us_per_input": round(tp * 1e3 / len(items), 2),
            "bit_exact": exact, "median_len": int(np.median(lens)),
            "autotune": {"sample_inputs": 512, "seconds": round(tune_s, 1),
                         "chosen": diff(asdict(best)) or "default",
                         "candidates": [{"tuning": diff(t) or "default", "ms": ms, "error": err}
                                        for t, ms, err in report]}}


def positions_leg(prog, data, n, dense_out, dev, steps=10, capacity=1 << 20):
    """The headline scan without output streams: match positions and counts only (the
    reference's consumers, bitgen/bitstream.py:27-67 and from_icgrep.py:600-611, read set-bit
    positions and counts).  Algorithmic bytes per launch: the input, 8 bytes per position and
    per count.  The positions must be exactly the set bits of the dense launch's streams."""
    import numpy as np
    import torch
    from bitgen_gb300.engine import bytes_input, out_layout

    inp = bytes_input(data)
    offs, words, total = out_layout([n])
    plan = prog.plan(inp, offs, total)
    pbuf = torch.empty(capacity, dtype=torch.int64, device=dev)
    counts = torch.empty((prog.n_outputs, 1), dtype=torch.int64, device=dev)
    plan.set_positions(pbuf)
    s = torch.cuda.current_stream(dev)
    sp = int(s.cuda_stream)
    for _ in range(3):
        plan.launch(data.data_ptr(), 0, counts.data_ptr(), sp)
    plan.sync(sp)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(steps):
        plan.launch(data.data_ptr(), 0, counts.data_ptr(), sp)
    e1.record(s)
    plan.sync(sp)
    ms = e0.elapsed_time(e1) / steps
    m = plan.positions_written(sp)
    got = np.sort(pbuf[:min(m, capacity)].cpu().numpy().view(np.uint64))
    plan.set_positions(None)
    # the dense launch's set bits, from its non-zero words
    W = (n + 31) // 32
    dv = dense_out[:, :W].view(torch.int32)
    nz = torch.nonzero(dv).cpu().numpy()
    vals = dv[nz[:, 0], nz[:, 1]].cpu().numpy().view(np.uint32)
    keys = []
    for (o, w), v in zip(nz.tolist(), vals.tolist()):
        for b in range(32):
            if (v >> (31 - b)) & 1 and 32 * w + b < n:
                keys.append((o << 52) | (32 * w + b))
    want = np.sort(np.array(keys, dtype=np.uint64))
    exact = bool(got.size == want.size and np.array_equal(got, want)
                 and int(counts.sum()) == want.size)
    peak, peak_kind = peaks()
    b_alg = n + 8 * int(m) + 8 * prog.n_outputs
    return {"GBps": round(n / ms / 1e6, 3), "ms": round(ms, 4), "steps": steps,
            "positions": int(m), "bit_exact_vs_dense_streams": exact,
            "roofline": {"bound": "hbm", "achieved": round(b_alg / ms / 1e6, 2), "peak": peak,
                         "unit": "GB/s", "frac": round(b_alg / ms / 1e6 / peak, 4),
                         "peak_kind": peak_kind, "algorithmic_bytes_per_launch": b_alg}}


def basis_hook_leg(gs, data, n, dense_out, dev, steps=10):
    """The reference runner's hook on the headline input: kernels/kernel_0.py written by
    write_kernel_module, imported the way from_icgrep.init_kernel does (bitgen/from_icgrep.py:
    169-193), its init_kernel(...)[3] = run_fn called on the basis planes the transpose hook
    made (bitgen/bitstream.py:166-225), as run_regex_kernel calls it (from_icgrep.py:575-582):
    one synchronous call per step.  The planes carry no bytes, so the classify pass rebuilds
    them for the q-gram filter.  Algorithmic bytes per call: the 8 planes (n bytes) plus each
    group's result stream.  The result must equal the headline launch's output streams."""
    import importlib
    import shutil
    import tempfile
    import torch
    from bitgen_gb300.backend import byte_stream_transpose, write_kernel_module

    npad = -(-n // 32) * 32
    bytestream = torch.zeros((1, 1, npad), dtype=torch.uint8, device=dev)
    bytestream[0, 0, :n].copy_(data)
    basis = torch.zeros((1, 1, 8, npad // 32), dtype=torch.uint32, device=dev)
    byte_stream_transpose(bytestream, basis)
    tmp = tempfile.mkdtemp(prefix="bg_hook_")
    try:
        write_kernel_module(gs, tmp)
        sys.path.insert(0, tmp)
        sys.modules.pop("kernels", None)
        sys.modules.pop("kernels.kernel_0", None)
        kmod = importlib.import_module("kernels.kernel_0")
        result, _, handle, run_fn, _ = kmod.init_kernel(len(gs), bytestream, basis, {})
    finally:
        if tmp in sys.path:
            sys.path.remove(tmp)
        shutil.rmtree(tmp, ignore_errors=True)
    for _ in range(3):
        run_fn(basis)
    s = torch.cuda.current_stream(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(steps):
        run_fn(basis)
    e1.record(s)
    torch.cuda.synchronize(dev)
    ms = e0.elapsed_time(e1) / steps
    W = npad // 32
    exact = bool(torch.equal(result[0, 0].view(torch.int32)[:, :W],
                             dense_out[:, :W].view(torch.int32)))
    handle.free()
    peak, peak_kind = peaks()
    b_alg = n + len(gs) * W * 4
    return {"GBps": round(n / ms / 1e6, 3), "ms": round(ms, 4), "steps": steps,
            "call": "kernels/kernel_0.init_kernel(...)[3](basis), synchronous",
            "bit_exact_vs_byte_launch": exact,
            "roofline": {"bound": "hbm", "achieved": round(b_alg / ms / 1e6, 2), "peak": peak,
                         "unit": "GB/s", "frac": round(b_alg / ms / 1e6 / peak, 4),
                         "peak_kind": peak_kind, "algorithmic_bytes_per_launch": b_alg}}


def transpose_leg(dev, n_bytes=1 << 30, reps=20, check_bytes=1 << 20, cpu_bytes=4 << 20):
    """The stand-alone transpose (the reference's byte_stream_transpose, kernel.cu:102-124):
    uint8 [1, 1, n] -> uint32 [1, 1, 8, n/32] on the device, 2n bytes of HBM traffic per call;
    the first `check_bytes` compared with the oracle's restatement of bitstream.py:228-258,
    which is also timed on the host over `cpu_bytes` (one thread, numpy)."""
    import numpy as np
    import torch
    from bitgen_gb300.engine import transpose
    from oracle.pablo_ref import transpose_ref

    g = torch.Generator(device=dev)
    g.manual_seed(6)
    src = torch.randint(0, 256, (1, 1, n_bytes), dtype=torch.uint8, device=dev, generator=g)
    dst = torch.empty((1, 1, 8, n_bytes // 32), dtype=torch.uint32, device=dev)
    s = torch.cuda.current_stream(dev)
    for _ in range(3):
        transpose(src, dst, s)
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(reps):
        transpose(src, dst, s)
    e1.record(s)
    torch.cuda.synchronize(dev)
    ms = e0.elapsed_time(e1) / reps
    head = src[0, 0, :check_bytes].cpu().numpy()
    want = transpose_ref(head)
    got = dst[0, 0, :, :check_bytes // 32].cpu().numpy()
    sample = src[0, 0, :cpu_bytes].cpu().numpy()
    t0 = time.perf_counter()
    transpose_ref(sample)
    cpu_s = time.perf_counter() - t0
    peak, peak_kind = peaks()
    return {"bytes": n_bytes, "reps": reps, "ms": round(ms, 4),
            "GBps": round(n_bytes / ms / 1e6, 3),
            "roofline": {"bound": "hbm", "achieved": round(2 * n_bytes / ms / 1e6, 2), "peak": peak,
                         "unit": "GB/s", "frac": round(2 * n_bytes / ms / 1e6 / peak, 4),
                         "peak_kind": peak_kind, "algorithmic_bytes_per_launch": 2 * n_bytes},
            "bit_exact_vs_oracle_first_bytes": check_bytes if np.array_equal(got, want) else False,
            "cpu_baseline": {"value": round(sample.size / cpu_s / 1e9, 6), "unit": "GB/s", "cores": 1,
                             "kind": "port", "sample": f"{sample.size} bytes, numpy restatement of "
                                                       f"bitstream.py:228-258, {cpu_s:.2f} s"}}


def dna_leg(dev, n_bytes, steps, check_bytes, ref_gpu=True):
    """64 IUPAC motifs (6-20 bases, every fourth split by a gap .{a,b}, 3 <= a <= 5, b <= a + 4) in 4 groups over DNA text
    (i.i.d. A/C/G/T, GC 42%, N runs, 80-column lines, 2^16 planted motif instances); per-group
    streams and counts, the program's default tuning (on a 4-letter text the q-gram filter
    passes nearly every tile, so the compiler picks the single-kernel form)."""
    import torch
    from bitgen_gb300 import workloads
    from bitgen_gb300.engine import Program, bytes_input, out_layout
    from bitgen_gb300.regex import compile_group

    t0 = time.perf_counter()
    ps = workloads.dna_motifs(64, seed=5)
    text = workloads.plant(workloads.dna_text(n_bytes, seed=6), ps.witnesses, 1 << 16, 7)
    gen_s = time.perf_counter() - t0
    groups = [compile_group(g) for g in ps.groups(4)]
    prog = Program(groups)
    data = torch.from_numpy(text).to(dev)
    inp = bytes_input(data)
    offs, words, total = out_layout([n_bytes])
    out = torch.empty((prog.n_outputs, total), dtype=torch.uint32, device=dev)
    counts = torch.empty((prog.n_outputs, 1), dtype=torch.int64, device=dev)
    plan = prog.plan(inp, offs, total)
    s = torch.cuda.current_stream(dev)
    sp = int(s.cuda_stream)
    for _ in range(3):
        plan.launch(data.data_ptr(), out.data_ptr(), counts.data_ptr(), sp)
    plan.sync(sp)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(steps):
        plan.launch(data.data_ptr(), out.data_ptr(), counts.data_ptr(), sp)
    e1.record(s)
    plan.sync(sp)
    ms = e0.elapsed_time(e1) / steps
    res = {"bytes": n_bytes, "regexes": len(ps.regexes), "groups": len(groups), "steps": steps,
           "GBps": round(n_bytes / ms / 1e6, 3), "ms": round(ms, 4),
           "form": "split" if prog.spec.n_parts else "single-kernel",
           "matches": int(counts.sum()), "text_gen_s": round(gen_s, 1)}
    if check_bytes is not None:
        check_bytes = min(check_bytes or n_bytes, n_bytes)
        cb, cpu_streams, cpu_counts = cpu_baseline(groups, text, check_bytes)
        if check_bytes == n_bytes:          # the streams and counts of the timed launches
            got, got_out = counts[:, 0].tolist(), out
        else:
            r = prog.scan(bytes_input(data[:check_bytes].contiguous()))
            got, got_out = r.counts[:, 0].tolist(), r.streams
        res["bit_exact_vs_cpu"] = {
            "bytes": check_bytes, "counts": [int(x) for x in got] == list(cpu_counts),
            "streams": streams_equal(got_out, cpu_streams, (check_bytes + 31) // 32)}
        del cpu_streams
        res["cpu_baseline"] = cb
    if ref_gpu:
        res["reference_gpu"] = reference_gpu_baseline(prog, ps.groups(4), data, dev)
    prog.close()
    del out, data
    return res


def popcounts(words):
    """Set bits per row of a device uint32 tensor [..., R, W] summed over the leading axes."""
    import torch
    x = words.reshape(-1, words.shape[-2], words.shape[-1]).view(torch.int32).to(torch.int64) \
        & 0xFFFFFFFF
    x = x - ((x >> 1) & 0x55555555)
    x = (x & 0x33333333) + ((x >> 2) & 0x33333333)
    x = (x + (x >> 4)) & 0x0F0F0F0F
    x = (x * 0x01010101 & 0xFFFFFFFF) >> 24
    return x.sum(dim=(0, 2)).tolist()


def reference_gpu_baseline(prog, groups, data, dev, target_s=0.25, guard_s=5.0):
    """The reference's own generated kernel (BitGen's KernelGenerated for these groups, made by
    oracle/ref_gpu.py with --pass-cc-advanced=0 --pass-short-circuit=0 --pass-graph-break=-1)
    timed on this GPU beside the engine, as a baseline.  One block scans one group over one
    whole input (grid = (groups, inputs), gen_cuda.py:409-411), so two forms are timed: one
    input (the runner's multi_input=1) and the input cut into 4 x SMs / groups inputs, the most
    blocks its grid can take.  Each form is calibrated on 1 MiB, then timed on a sample sized
    for about `target_s` per launch; a form whose calibration launch takes over `guard_s` is
    not timed further.  The streams of the one-input form and the counts of both are compared
    with this engine's on the same bytes."""
    import torch
    from oracle import ref_gpu
    from bitgen_gb300.backend import byte_stream_transpose
    from bitgen_gb300.engine import bytes_input, pack_bytes

    if not ref_gpu.available(ref_gpu.DNA):
        return {"unavailable": "generated kernel absent (oracle/ref_gpu.py makes it where the "
                               "reference tree is)"}
    k = ref_gpu.RefKernel(ref_gpu.DNA, groups)
    s = torch.cuda.current_stream(dev)
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    rec = {"kernel": "BitGen KernelGenerated (bitgen/codegen/gen_cuda.py) from this project's "
                     "Pablo, --pass-cc-advanced=0 --pass-short-circuit=0 --pass-graph-break=-1",
           "block": k.block}

    def run(n_bytes, inputs, reps):
        words = n_bytes // 32 // inputs
        flat, basis = k.basis_buffer(inputs, words, dev)
        byte_stream_transpose(data[:inputs * words * 32].view(1, inputs, words * 32), basis)
        res = torch.zeros((inputs, k.groups, words), dtype=torch.uint32, device=dev)
        k.launch(flat, inputs, words, res, s)                       # the checked result
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        for _ in range(reps):
            k.launch(flat, inputs, words, res, s)
        e1.record(s)
        torch.cuda.synchronize(dev)
        return e0.elapsed_time(e1) / reps, res, words

    for form, inputs in (("one_input", 1), ("filled", max(1, 4 * sms // k.groups))):
        unit = 32 * inputs
        t0 = time.perf_counter()
        ms1, _, _ = run(-(-(1 << 20) // unit) * unit, inputs, 1)
        if time.perf_counter() - t0 > guard_s:
            rec[form] = {"skipped": f"1 MiB calibration launch took over {guard_s} s"}
            continue
        n = int(min(data.numel(), (1 << 20) * target_s * 1e3 / max(ms1, 1e-3))) // unit * unit
        ms, res, words = run(n, inputs, 3)
        got = popcounts(res)
        sub = data[:inputs * words * 32]
        if inputs == 1:
            r = prog.scan(bytes_input(sub.contiguous()))
            want = r.counts[:, 0].tolist()
            eq = {"streams_equal": bool(torch.equal(res[0], r.streams[:, :words]))}
        else:
            r = prog.scan(pack_bytes(list(sub.view(inputs, words * 32)), device=dev))
            want = r.counts.sum(dim=1).tolist()
            eq = {}
        rec[form] = {"grid": [k.groups, inputs], "bytes": inputs * words * 32, "ms": round(ms, 3),
                     "GBps": round(inputs * words * 32 / ms / 1e6, 3),
                     "counts_equal": [int(x) for x in got] == [int(x) for x in want], **eq}
        del res, r
    return rec


def served_leg(dev, n_req, probe_req=3000, plain_req=1000, arena_bytes=1 << 30):
    """Served configuration: Poisson arrivals (seed 8) of `n_req` requests, lengths log-uniform
    64 B - 4 MiB, each against one of three resident pattern sets (32, 256, 1024 regexes),
    admitted by a 120 GB HBM budget; continuous batching vs one launch per request.

    Payloads are seeded printable text with planted matches in one pinned arena per pattern set
    (each set's requests back to back in arrival order, so a batch is one copy).  The Poisson
    rate is 80% of the served capacity measured first by a saturation probe (the first
    `probe_req` requests, all available at once, timed on the second of two passes).  The plain form is timed on the first
    `plain_req` requests (all available at once) and its counts compared with the served
    results of those requests."""
    import numpy as np
    import torch
    from bitgen_gb300 import workloads
    from bitgen_gb300.engine import Program
    from bitgen_gb300.regex import compile_group
    from bitgen_gb300.served import Request, RequestArena, Server, latency_stats, serve_plain

    sets, arenas = {}, {}
    for name, n, seed in (("p32", 32, 81), ("p256", 256, 3), ("p1024", 1024, 83)):
        ps = workloads.throughput_patterns(seed=seed, n=n)
        sets[name] = (ps, Program([compile_group(g) for g in ps.groups(min(16, max(1, n // 16)))]))
        base = workloads.plant(workloads.printable_text(16 << 20, seed + 1000), ps.witnesses, 4096,
                               seed + 2000)
        arenas[name] = RequestArena(arena_bytes, fill=base)
    names = list(sets)
    progs = {k: v[1] for k, v in sets.items()}

    def requests(count, rate):
        for a in arenas.values():
            a.at = 0
        arr, lens, which = workloads.served_requests(count, seed=8, rate_per_s=rate)
        return [Request(i, float(arr[i]), names[int(which[i])],
                        arenas[names[int(which[i])]].take(int(lens[i]))) for i in range(count)], lens

    def server():
        return Server(progs, hbm_budget=120 << 30, slots=4, max_batch_bytes=64 << 20,
                      max_batch_inputs=256, arenas=list(arenas.values()))

    # saturation probe: every request available at once, timed on its second pass (the first
    # loads every program's kernels and touches every plan and staging buffer)
    probe, plens = requests(min(probe_req, n_req), 1e12)
    srv = server()
    srv.serve(probe, realtime=False)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    srv.serve(probe, realtime=False)
    cap_s = time.perf_counter() - t0
    capacity = len(probe) / cap_s                 # requests per second
    rate = 0.8 * capacity
    reqs, lens = requests(n_req, rate)
    total = int(lens.sum())
    t0 = time.perf_counter()
    got = srv.serve(reqs, realtime=True)
    span = time.perf_counter() - t0
    sample = reqs[:min(plain_req, n_req)]
    serve_plain(progs, sample[:200], realtime=False, arenas=list(arenas.values()))   # warm
    t1 = time.perf_counter()
    plain = serve_plain(progs, sample, realtime=False, arenas=list(arenas.values()))
    pspan = time.perf_counter() - t1
    exact = all(np.array_equal(got[r.rid].counts, plain[r.rid].counts) for r in sample)
    ptotal = int(sum(r.data.size for r in sample))
    served_GBps = total / span / 1e9
    plain_GBps = ptotal / pspan / 1e9
    return {"requests": n_req, "bytes": total, "arrivals": "poisson (seed 8)",
            "capacity_probe": {"requests": len(probe), "GBps": round(int(plens.sum()) / cap_s / 1e9, 3),
                               "req_per_s": round(capacity, 1)},
            "offered_rate_per_s": round(rate, 1), "offered_load": "80% of the probed capacity",
            "pattern_sets": {k: len(v[0].regexes) for k, v in sets.items()},
            "served": {**{k: round(v, 3) for k, v in latency_stats(got).items() if k != "n"},
                       "GBps": round(served_GBps, 3), "wall_s": round(span, 2)},
            "plain": {"requests": len(sample), "GBps": round(plain_GBps, 3),
                      "form": "one launch per request, all available at once"},
            "served_over_plain": round(served_GBps / plain_GBps, 2),
            "counts_equal_plain": exact, "hbm_budget_GB": 120,
            "payloads": "pinned arena per pattern set (1 GiB, seeded text, planted matches)"}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    ps, groups, base, reps = workload(args)
    vals = []
    for i in range(args.warmup + args.steps):
        cb, _, _ = cpu_baseline(groups, base, args.cpu_sample or args.bytes)
        if i >= args.warmup:
            vals.append(cb["value"])
    v = statistics.median(vals)
    cb["value"] = v
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic (seeded)",
            "config": {"workload": f"throughput: {args.regexes} synthetic regexes, {args.groups} groups, "
                                   f"CPU sample of {args.cpu_sample or args.bytes} bytes"},
            "cpu_baseline": cb,
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)

    import numpy as np
    import torch
    import torch.distributed as dist

    if args.served_only:
        print(json.dumps(served_leg(torch.device("cuda", 0), args.served_requests)), flush=True)
        return

    if args.dna_only:
        print(json.dumps(dna_leg(torch.device("cuda", 0), args.dna_bytes, max(1, args.steps),
                                 None if args.no_cpu else args.cpu_sample,
                                 ref_gpu=not args.no_ref_gpu)), flush=True)
        return

    from bitgen_gb300.compiler import Tuning
    from bitgen_gb300.engine import Program, bytes_input, out_layout
    from bitgen_gb300.regex import compile_group

    from bitgen_gb300 import replicas
    _, world, local = replicas.world()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    rank, world = replicas.init("nccl", dev)

    ps, groups, base, reps = workload(args)
    gs = [compile_group(g) for g in groups]
    tuning = Tuning(wpt=args.wpt) if args.wpt else Tuning()
    t0 = time.perf_counter()
    prog = Program(gs, tuning=tuning)
    compile_s = time.perf_counter() - t0
    n = args.bytes
    host = torch.from_numpy(np.tile(base, reps)[:n].copy()).pin_memory()
    data = host.to(dev)
    inp = bytes_input(data)
    offs, words, total = out_layout([n])
    out = torch.empty((prog.n_outputs, total), dtype=torch.uint32, device=dev)
    counts = torch.empty((prog.n_outputs, 1), dtype=torch.int64, device=dev)
    plan = prog.plan(inp, offs, total)
    stream = torch.cuda.current_stream(dev)
    sp = int(stream.cuda_stream)

    def step():
        plan.launch(data.data_ptr(), out.data_ptr(), counts.data_ptr(), sp)

    for _ in range(max(3, args.warmup)):
        step()
    plan.sync(sp)
    # bit-exact self-check of this very configuration against the CPU evaluator (rank 0, sample)
    check = None
    if rank == 0 and not args.no_cpu:
        sample = min(args.cpu_sample or n, n)
        cb, cpu_streams, cpu_counts = cpu_baseline(groups, base, sample)
        if sample == n:                     # the streams and counts of the warm-up launches
            gpu_counts, gpu_out = [int(x) for x in counts[:, 0].tolist()], out
        else:
            r = prog.scan(bytes_input(data[:sample].contiguous()))
            gpu_counts, gpu_out = [int(x) for x in r.counts[:, 0].tolist()], r.streams
        check = {"bytes": sample, "counts": gpu_counts == list(cpu_counts),
                 "streams": streams_equal(gpu_out, cpu_streams, (sample + 31) // 32)}
        del cpu_streams
    else:
        cb = None

    replicas.barrier()
    torch.cuda.synchronize(dev)
    clocks = Clocks(local)
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        step()
    ev1.record(stream)
    torch.cuda.synchronize(dev)
    plan.sync(sp)
    replicas.barrier()
    clk = clocks.stop()
    ms = ev0.elapsed_time(ev1) / args.steps
    # per-launch time of one scan (prologue, carry pre-pass and carry scan when the program has
    # them, main kernel: all on `stream`) for the roofline
    k0 = torch.cuda.Event(enable_timing=True)
    k1 = torch.cuda.Event(enable_timing=True)
    kt, wall = [], []
    for _ in range(10):
        t0 = time.perf_counter()
        k0.record(stream)
        step()
        k1.record(stream)
        torch.cuda.synchronize(dev)
        wall.append((time.perf_counter() - t0) * 1e3)
        kt.append(k0.elapsed_time(k1))
    kernel_ms = statistics.median(kt)
    # the reference runner's own measure: host clock around launch + synchronize, averaged
    avg_ms_sync = statistics.mean(wall)
    # work counters of the last launch (read back after the timed region)
    st = plan.stats(sp)
    work = {"form": st["form"], "tiles": st["tiles"]}
    if st["form"] == "split":
        work.update(parts=len(st["tiles_run"]), rows_listed=sum(st["rows"]),
                    part_runs_per_tile=round(sum(st["tiles_run"]) / max(1, st["tiles"]), 4))

    # end to end through the public API: pinned host bytes in, counts out, every step.  Serial:
    # copy, scan, read back one after another on one stream.  Streamed (StreamScanner, the
    # headline): the copy of step i + 1 runs on copy streams while step i is scanned.
    e2e_steps = max(3, min(args.steps, 10))
    h_counts = torch.empty((prog.n_outputs, 1), dtype=torch.int64).pin_memory()
    torch.cuda.synchronize(dev)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(e2e_steps):
        data.copy_(host, non_blocking=True)
        step()
        h_counts.copy_(counts, non_blocking=True)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    serial_ms = e0.elapsed_time(e1) / e2e_steps
    from bitgen_gb300.streaming import StreamScanner
    sc = StreamScanner(prog, n, dev, copy_streams=2)
    for _ in range(2):
        sc.submit(host)
    sc.synchronize()
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    handles = [sc.submit(host) for _ in range(e2e_steps)]
    sc.synchronize()
    e2e_ms = (time.perf_counter() - t0) * 1e3 / e2e_steps
    streamed_counts = sc.counts(handles[-1])
    streamed_exact = streamed_counts == [int(x) for x in h_counts[:, 0].tolist()]

    ms, kernel_ms, e2e_ms, serial_ms = replicas.max_over_ranks([ms, kernel_ms, e2e_ms, serial_ms],
                                                               device=dev)
    total_bytes = n * world
    value = total_bytes / (ms / 1e3) / 1e9
    peak, peak_kind = peaks()
    b_alg = n + prog.n_outputs * ((n + 31) // 32) * 4   # input once + each output stream once
    achieved = b_alg / (kernel_ms / 1e3) / 1e9
    info = prog.info()
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
        "data": "synthetic (seeded regexes and printable-ASCII text)",
        "config": {"workload": f"throughput: {args.regexes} synthetic regexes in {len(gs)} groups over "
                               f"{n >> 20} MiB printable ASCII (1 MiB tiled), per-group match streams + counts",
                   "regexes": args.regexes, "groups": len(gs), "input_bytes": n,
                   "parallelism": f"replicas x{world}", "l2": "input larger than L2 (no flush)",
                   "tuning": {"wpt": info.get("wpt"), "halo_lanes": info.get("halo_lanes"),
                              "block": tuning.block, "skip_interval": tuning.skip_interval},
                   "registers": info.get("registers"), "adds": info.get("adds"),
                   "pre_pass_adds": info.get("pre_adds"),
                   "compile_s": round(compile_s, 2), "bit_exact_vs_cpu": check,
                   "work": work},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 2), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 5), "traffic": None,
                     "peak_kind": peak_kind, "algorithmic_bytes_per_launch": b_alg,
                     "kernel_ms": round(kernel_ms, 4), "kernel_ms_of": "median of 10 launches",
                     "avg_ms_sync": round(avg_ms_sync, 4)},
        "e2e": {"value": round(total_bytes / (e2e_ms / 1e3) / 1e9, 3), "unit": UNIT,
                "h2d_bytes_per_step": n, "d2h_bytes_per_step": prog.n_outputs * 8,
                "mode": "streamed (StreamScanner: copy of step i+1 beside the scan of step i, "
                        "wall clock over the steps)",
                "counts_equal_serial": streamed_exact,
                "serial_value": round(total_bytes / (serial_ms / 1e3) / 1e9, 3)},
        "gpu_launches": info.get("kernels_per_scan", 0) * args.steps,
        "clocks": clk,
    }
    if cb is not None:
        line["cpu_baseline"] = cb
    if rank == 0 and prog.spec.n_parts:
        try:
            line["positions_only"] = positions_leg(prog, data, n, out, dev)
        except Exception as e:
            line["positions_only"] = {"error": f"{type(e).__name__}: {e}"[:300]}
    if rank == 0 and n % 32 == 0:
        try:
            line["basis_hook"] = basis_hook_leg(gs, data, n, out, dev)
        except Exception as e:
            line["basis_hook"] = {"error": f"{type(e).__name__}: {e}"[:300]}
    if rank == 0 and not args.no_modes:
        try:
            line["batched"] = batched_leg(prog, gs, ps, dev)
        except Exception as e:  # a failed leg is reported, it does not void the main line
            line["batched"] = {"error": f"{type(e).__name__}: {e}"[:300]}
        try:
            line["transpose"] = transpose_leg(dev)
        except Exception as e:
            line["transpose"] = {"error": f"{type(e).__name__}: {e}"[:300]}
        try:
            line["dna"] = dna_leg(dev, args.dna_bytes, 5, None if args.no_cpu else args.cpu_sample)
        except Exception as e:
            line["dna"] = {"error": f"{type(e).__name__}: {e}"[:300]}
        try:
            line["served"] = served_leg(dev, args.served_requests)
        except Exception as e:
            line["served"] = {"error": f"{type(e).__name__}: {e}"[:300]}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist.is_initialized():
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
