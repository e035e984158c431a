"""Python host API of the engine: compile a pattern set once, scan device inputs with it.

``Program`` owns one compiled pattern set.  Straight-line programs (the common case, and every
program whose loops are MatchStar loops) become one fused NVRTC kernel driven through launch
plans; programs that keep other ``while`` / ``if`` blocks run on the native whole-stream
executor.  Both are reached only through the C ABI of ``libbitgen_gb300.so``; there is no
CPU path.

Inputs are device ``uint8`` tensors (raw bytes, transposed inside the kernel) or device
``uint32`` basis tensors in the reference layout.  Outputs are ``uint32`` streams in the
reference bit layout (character ``32w + j`` at bit ``31 - j`` of word ``w``) and ``int64``
match counts.
"""

from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass
from typing import Dict, List, Optional, Sequence, Tuple

import torch

from . import _native as N
from .compiler import NotFusable, Tuning, build_dag, fusable, generate_kernel, convert_star_loops
from .pablo import Group, If, Op, While
from .regex import compile_group

_DEFAULT_CACHE = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), ".bg_cache")


def _ensure_cache_dir():
    d = os.environ.get("BG_CACHE_DIR")
    if d is None:
        d = _DEFAULT_CACHE
        os.environ["BG_CACHE_DIR"] = d
    if d:
        os.makedirs(d, exist_ok=True)


def _i64(values) -> C.Array:
    vals = list(int(v) for v in values)
    return (C.c_int64 * max(1, len(vals)))(*vals)


def _stream_ptr(stream: Optional[torch.cuda.Stream]) -> int:
    s = stream if stream is not None else torch.cuda.current_stream()
    return int(s.cuda_stream)


# ----------------------------------------------------------------------------------------
# whole-stream executor lowering
# ----------------------------------------------------------------------------------------
_IOP = {"and": 0, "or": 1, "xor": 2, "not": 3, "sel": 4, "advance": 5, "matchstar": 6,
        "scanthru": 7, "assign": 8, "lookahead": 11}
OP_WHILE, OP_IF = 9, 10


def lower_interp(groups: Sequence[Group], per_regex: bool = False):
    """Flatten Pablo groups into the executor's instruction list (see ``bitgen_gb300.h``).

    Variables get slots by linear-scan allocation over their live ranges; a variable referenced
    inside a loop stays live for the whole loop.  A destination never shares a slot with an
    operand of the same instruction (Advance cannot run in place).
    Returns ``(code, n_slots, output_slots)``."""
    flat: List[list] = []        # [op, dst, a, b, c, shift] with variable names
    loops: List[Tuple[int, int]] = []
    outs_v: List[str] = []

    def name(x, gi):
        if x in ("0", "1") or (x.startswith("basis") and x[5:].isdigit() and len(x) == 6):
            return x
        return f"g{gi}:{x}"

    def emit(stmts, gi):
        for s_ in stmts:
            if isinstance(s_, Op):
                a = [name(x, gi) for x in s_.args] + [None, None, None]
                flat.append([_IOP[s_.op], name(s_.dst, gi), a[0], a[1], a[2], s_.shift])
            elif isinstance(s_, While):
                at = len(flat)
                flat.append([OP_WHILE, None, name(s_.cond, gi), None, None, 0])
                emit(s_.body, gi)
                flat[at][5] = len(flat) - at - 1
                loops.append((at, len(flat) - 1))
            else:
                at = len(flat)
                flat.append([OP_IF, None, name(s_.cond, gi), None, None, 0])
                emit(s_.then, gi)
                nthen = len(flat) - at - 1
                emit(s_.orelse or [], gi)
                flat[at][5] = nthen
                flat[at][3] = len(flat) - at - 1 - nthen   # else length (stored in b)

    for gi, g in enumerate(groups):
        emit(convert_star_loops(g.stmts), gi)
        if per_regex and g.regex_results:
            outs_v.extend(name(r, gi) for r in g.regex_results)
        else:
            outs_v.append(name(g.result, gi))

    fixed = {f"basis{i}": i for i in range(8)}
    fixed["0"] = 8
    fixed["1"] = 9
    first: Dict[str, int] = {}
    last: Dict[str, int] = {}
    for i, ins in enumerate(flat):
        refs = [ins[1], ins[2]] + ([ins[3]] if ins[0] != OP_IF else []) + [ins[4]]
        for v in refs:
            if v is None or v in fixed:
                continue
            first.setdefault(v, i)
            last[v] = i
    for lo, hi in loops:
        for v in list(first):
            if first[v] <= hi and last[v] >= lo:
                first[v] = min(first[v], lo)
                last[v] = max(last[v], hi)
    end = len(flat)
    for v in outs_v:
        if v not in fixed:
            first.setdefault(v, 0)
            last[v] = end
    order = sorted(first, key=lambda v: (first[v], v))
    free: List[int] = []
    active: List[Tuple[int, str]] = []
    slot_of: Dict[str, int] = dict(fixed)
    n_slots = 10
    import heapq
    for v in order:
        st = first[v]
        while active and active[0][0] < st:
            _, dead = heapq.heappop(active)
            heapq.heappush(free, slot_of[dead])
        if free:
            sl = heapq.heappop(free)
        else:
            sl = n_slots
            n_slots += 1
        slot_of[v] = sl
        heapq.heappush(active, (last[v], v))

    def S(v):
        return -1 if v is None else slot_of[v]

    code = []
    for ins in flat:
        op = ins[0]
        if op == OP_IF:
            code.append((op, -1, S(ins[2]), ins[3], -1, ins[5]))
        elif op == OP_WHILE:
            code.append((op, -1, S(ins[2]), -1, -1, ins[5]))
        else:
            code.append((op, S(ins[1]), S(ins[2]), S(ins[3]), S(ins[4]), ins[5]))
    return code, n_slots, [slot_of[v] for v in outs_v]


# ----------------------------------------------------------------------------------------
# layouts and results
# ----------------------------------------------------------------------------------------
@dataclass
class Inputs:
    """Device inputs of one scan: a flat buffer plus per-input offsets and lengths."""
    data: torch.Tensor          # uint8 bytes or uint32 basis words (device)
    kind: int                   # N.BG_INPUT_BYTES / N.BG_INPUT_BASIS
    offsets: List[int]          # byte offsets (bytes) / word offset of plane 0 (basis)
    lengths: List[int]          # characters per input
    basis_stride: int = 0       # words between planes (basis)

    @property
    def n(self) -> int:
        return len(self.lengths)


def pack_bytes(items: Sequence, device="cuda", align: int = 32) -> Inputs:
    """Pack byte strings / uint8 arrays / tensors into one aligned device buffer."""
    offs, lens, chunks = [], [], []
    pos = 0
    for it in items:
        if isinstance(it, torch.Tensor):
            t = it.reshape(-1).to(torch.uint8)
        else:
            import numpy as np
            t = torch.from_numpy(np.frombuffer(bytes(it), dtype=np.uint8).copy())
        offs.append(pos)
        lens.append(int(t.numel()))
        chunks.append(t)
        pos += -(-int(t.numel()) // align) * align
    buf = torch.zeros(max(pos, align), dtype=torch.uint8, device=device)
    for o, t in zip(offs, chunks):
        if t.numel():
            buf[o:o + t.numel()].copy_(t.to(device, non_blocking=True))
    return Inputs(buf, N.BG_INPUT_BYTES, offs, lens)


def bytes_input(t: torch.Tensor) -> Inputs:
    """One device uint8 tensor as a single input (no copy)."""
    assert t.is_cuda and t.dtype == torch.uint8 and t.is_contiguous()
    return Inputs(t.reshape(-1), N.BG_INPUT_BYTES, [0], [t.numel()])


def basis_input(basis: torch.Tensor, n_chars: Optional[Sequence[int]] = None) -> Inputs:
    """Reference basis tensor ``uint32 [S=1, M, 8, W]`` (or ``[M, 8, W]``) as M inputs."""
    b = basis.reshape(-1, 8, basis.shape[-1])
    M, _, W = b.shape
    lens = list(n_chars) if n_chars is not None else [32 * W] * M
    return Inputs(b.reshape(-1), N.BG_INPUT_BASIS, [m * 8 * W for m in range(M)], lens, W)


@dataclass
class ScanResult:
    streams: Optional[torch.Tensor]   # uint32 [n_outputs, total_words]
    counts: Optional[torch.Tensor]    # int64 [n_outputs, n_inputs]
    word_offsets: List[int]
    words: List[int]
    positions: Optional["np.ndarray"] = None  # sorted u64 (output << 52 | input << 32 | pos)
    stats: Optional[dict] = None  # work counters (scan(stats=True); None on the whole-stream executor)

    def stream(self, output: int, input_index: int = 0) -> torch.Tensor:
        o = self.word_offsets[input_index]
        return self.streams[output, o:o + self.words[input_index]]

    def match_positions(self, output: int, input_index: int = 0):
        """Sorted match-end positions of one output over one input (sparse output)."""
        import numpy as np
        key = (np.uint64(output) << np.uint64(52)) | (np.uint64(input_index) << np.uint64(32))
        lo = np.searchsorted(self.positions, key)
        hi = np.searchsorted(self.positions, key + np.uint64(1 << 32))
        return (self.positions[lo:hi] & np.uint64(0xFFFFFFFF)).astype(np.int64)


def out_layout(lengths: Sequence[int], align_words: int = 4) -> Tuple[List[int], List[int], int]:
    offs, words = [], []
    pos = 0
    for n in lengths:
        W = -(-int(n) // 32)
        offs.append(pos)
        words.append(W)
        pos += -(-W // align_words) * align_words
    return offs, words, max(pos, 1)


class Plan:
    """A launch plan: device tables + look-back records for an input layout.

    ``Plan(program, inp, ...)`` binds one fixed layout; ``Plan.reserve(...)`` makes a plan with
    room for changing layouts set by :meth:`set_layout` (batched / served scans)."""

    def __init__(self, program: "Program", inp: Optional[Inputs], out_offsets: Sequence[int] = (),
                 out_stride: int = 0, _handle=None):
        self.program = program
        self._scratch: Optional[torch.Tensor] = None
        self.out_stride = out_stride
        self._device = None
        if _handle is not None:
            self._h = _handle
            self.n_inputs = 0
            return
        self.n_inputs = inp.n
        self._device = inp.data.device
        lay = N.Layout(inp.kind, inp.n, _i64(inp.offsets), _i64(inp.lengths), inp.basis_stride,
                       _i64(out_offsets), out_stride)
        h = C.c_void_p()
        N.check(N.lib().bg_plan_create(program._handle, C.byref(lay), C.byref(h)), "bg_plan_create")
        self._h = h

    @classmethod
    def reserve(cls, program: "Program", kind: int, max_inputs: int, max_tiles: int) -> "Plan":
        h = C.c_void_p()
        N.check(N.lib().bg_plan_reserve(program._handle, kind, max_inputs, max_tiles, C.byref(h)),
                "bg_plan_reserve")
        return cls(program, None, _handle=h)

    def set_layout(self, inp: Inputs, out_offsets: Sequence[int], out_stride: int, stream: int):
        lay = N.Layout(inp.kind, inp.n, _i64(inp.offsets), _i64(inp.lengths), inp.basis_stride,
                       _i64(out_offsets), out_stride)
        N.check(N.lib().bg_plan_set_layout(self._h, C.byref(lay), stream), "bg_plan_set_layout")
        self.n_inputs = inp.n
        self.out_stride = out_stride
        self._device = inp.data.device

    def _ensure_scratch(self):
        """A program that merges outputs across parts needs output streams on every launch;
        counts-only launches write into this plan-owned buffer, made on the first of them (so
        before any graph capture that replays the launch)."""
        need = self.program.n_outputs * max(1, self.out_stride)
        if self._scratch is None or self._scratch.numel() < need:
            self._scratch = torch.empty(need, dtype=torch.uint32, device=self._device)

    @property
    def tiles(self) -> int:
        return int(N.lib().bg_plan_tiles(self._h))

    def set_positions(self, buf: Optional[torch.Tensor], count_capacity: int = 0):
        """Sparse output buffer (int64 view of u64 entries) for later launches, or None.  A
        program whose parts share outputs can then also be launched without output streams
        (positions only): its position set holds twice the buffer's entries.  With no buffer,
        ``count_capacity`` > 0 sizes that set for counts-only launches."""
        ptr, cap = (buf.data_ptr(), buf.numel()) if buf is not None else (None, int(count_capacity))
        N.check(N.lib().bg_plan_set_positions(self._h, ptr, cap), "bg_plan_set_positions")
        self._set_capacity = cap

    def positions_written(self, stream: int) -> int:
        v = C.c_int64()
        N.check(N.lib().bg_plan_positions_written(self._h, stream, C.byref(v)), "bg_plan_positions_written")
        return int(v.value)

    def stats(self, stream: int) -> dict:
        """Work counters of the last launch (waits for `stream`), the counterpart of the
        reference's optional ``dyn_stats`` buffer: the tiles of the launch and, for a split-form
        program, per part the tiles the execute pass ran it on (``tiles_run``), the 32-tile rows
        of its work list (``rows``) and the outputs it writes (``part_outputs``).  A
        single-kernel program runs every term on every tile."""
        spec = self.program.spec
        st = {"form": "split" if spec.n_parts else "single-kernel", "tiles": self.tiles}
        if spec.n_parts:
            k = spec.n_parts
            tiles_run, rows = (C.c_int64 * k)(), (C.c_int64 * k)()
            N.check(N.lib().bg_plan_stats(self._h, stream, k, tiles_run, rows), "bg_plan_stats")
            st.update(tiles_run=list(tiles_run), rows=list(rows),
                      part_outputs=[list(o) for o in spec.part_outputs])
        return st

    def set_wait_limit(self, cycles: int, debug_wait_tile: int = -1):
        N.check(N.lib().bg_plan_set_wait_limit(self._h, cycles, debug_wait_tile), "bg_plan_set_wait_limit")

    def launch(self, data_ptr: int, out_ptr: int, counts_ptr: int, stream: int):
        if not out_ptr and self.program.merges and not getattr(self, "_set_capacity", 0):
            self._ensure_scratch()
            out_ptr = self._scratch.data_ptr()
        N.check(N.lib().bg_plan_launch(self._h, data_ptr, out_ptr or None, counts_ptr or None,
                                       stream), "bg_plan_launch")

    def sync(self, stream: int):
        N.check(N.lib().bg_plan_sync(self._h, stream), "bg_plan_sync")

    def close(self):
        if getattr(self, "_h", None):
            N.lib().bg_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Program:
    """A compiled pattern set (one or more Pablo groups)."""

    def __init__(self, groups: Sequence[Group], per_regex: bool = False,
                 tuning: Optional[Tuning] = None, executor: str = "auto", name: str = "bg_scan"):
        self.groups = list(groups)
        self.per_regex = per_regex
        self.tuning = tuning or Tuning()
        lib = N.lib()
        fuse = executor == "fused" or (executor == "auto" and all(fusable(g) for g in self.groups))
        if executor == "fused" and not all(fusable(g) for g in self.groups):
            raise NotFusable("program keeps while/if blocks")
        self.fused = fuse
        self._handle = None
        self._interp = None
        self._plans: Dict[tuple, Plan] = {}
        if fuse:
            try:
                self.spec = generate_kernel(self.groups, self.tuning, per_regex, name)
            except NotFusable:
                if executor == "fused":
                    raise
                fuse = False
        self.fused = fuse
        self.merges = bool(fuse and self.spec.merges)
        if fuse:
            _ensure_cache_dir()
            self.n_outputs = self.spec.n_outputs
            src = self.spec.source.encode()
            self._desc = N.KernelDesc(src, len(src), name.encode(), self.spec.n_outputs,
                                      self.spec.n_adds, self.spec.halo_lanes, self.spec.wpt,
                                      self.spec.block, self.spec.tail_lanes, self.spec.n_pre,
                                      self.spec.n_run,
                                      N.BG_PROGRAM_MERGES if self.spec.merges else 0,
                                      self.spec.n_parts)
            h = C.c_void_p()
            N.check(lib.bg_program_create(C.byref(self._desc), C.byref(h)), "bg_program_create")
            self._handle = h
        else:
            self.spec = None
            code, n_slots, outs = lower_interp(self.groups, per_regex)
            arr = (N.Instr * max(1, len(code)))(*[N.Instr(*c) for c in code])
            oarr = (C.c_int32 * max(1, len(outs)))(*outs)
            h = C.c_void_p()
            N.check(lib.bg_interp_create(arr, len(code), n_slots, oarr, len(outs), C.byref(h)),
                    "bg_interp_create")
            self._interp = h
            self.n_outputs = len(outs)

    @classmethod
    def from_regex_groups(cls, regex_groups: Sequence[Sequence[str]], matchstar: bool = True, **kw):
        return cls([compile_group(list(g), matchstar=matchstar) for g in regex_groups], **kw)

    # ---------------------------------------------------------------------------------
    def info(self) -> dict:
        if not self.fused:
            return {"executor": "whole-stream"}
        r, l, b = C.c_int32(), C.c_int32(), C.c_int32()
        N.check(N.lib().bg_program_info(self._handle, C.byref(r), C.byref(l), C.byref(b)), "bg_program_info")
        return {"executor": "fused", "registers": r.value, "local_bytes": l.value,
                "blocks_per_sm": b.value, "halo_lanes": self.spec.halo_lanes, "wpt": self.spec.wpt,
                "adds": self.spec.n_adds, "pre_adds": self.spec.n_pre, "outputs": self.spec.n_outputs,
                "form": "split" if self.spec.n_parts else "single-kernel",
                "kernels_per_scan": self.kernels_per_scan()}

    def kernels_per_scan(self) -> int:
        """Kernels one ``Plan.launch`` starts: in the split form classify (which also does the
        launch prologue), the row kernel (carry scan and work list) and execute; else the
        prologue, the pre-pass and carry scan (with pre-pass additions) and the main kernel."""
        if self.spec.n_parts:
            return 3
        return 1 + 1 + 2 * int(self.spec.n_pre > 0)

    def tiles_for(self, lengths: Sequence[int]) -> int:
        """Tiles one launch over inputs of these lengths needs."""
        tw = self.spec.tile_words
        return sum(max(1, -(-(-(-int(n) // 32)) // tw)) for n in lengths)

    def plan(self, inp: Inputs, out_offsets: Sequence[int], out_stride: int) -> Plan:
        key = (inp.kind, tuple(inp.offsets), tuple(inp.lengths), inp.basis_stride,
               tuple(out_offsets), out_stride)
        p = self._plans.get(key)
        if p is None:
            p = Plan(self, inp, out_offsets, out_stride)
            self._plans[key] = p
        return p

    def scan(self, inp: Inputs, streams: bool = True, counts: bool = True,
             out: Optional[torch.Tensor] = None, out_offsets: Optional[Sequence[int]] = None,
             out_stride: Optional[int] = None, stream: Optional[torch.cuda.Stream] = None,
             sync: bool = True, max_iterations: Optional[int] = None,
             positions: bool = False, pos_capacity: int = 1 << 22, stats: bool = False) -> ScanResult:
        dev = inp.data.device
        if out_offsets is None:
            offs, words, total = out_layout(inp.lengths)
        else:
            offs = list(out_offsets)
            words = [-(-int(n) // 32) for n in inp.lengths]
            total = out_stride
        if streams and out is None:
            out = torch.empty((self.n_outputs, total), dtype=torch.uint32, device=dev)
        cnt = torch.empty((self.n_outputs, inp.n), dtype=torch.int64, device=dev) if counts else None
        sp = _stream_ptr(stream)
        out_ptr = out.data_ptr() if streams else 0
        cnt_ptr = cnt.data_ptr() if counts else 0
        stride = out_stride if out_stride is not None else total
        pos = st = None
        if self.fused:
            plan = self.plan(inp, offs, stride)
            pbuf = torch.empty(pos_capacity, dtype=torch.int64, device=dev) if positions else None
            # positions without streams: a program whose parts share outputs counts each bit
            # once through the plan's position set instead of the output streams
            plan.set_positions(pbuf)
            plan.launch(inp.data.data_ptr(), out_ptr, cnt_ptr, sp)
            if sync or positions:
                plan.sync(sp)
            if positions:
                import numpy as np
                n = plan.positions_written(sp)
                pos = np.sort(pbuf[:min(n, pos_capacity)].cpu().numpy().view(np.uint64))
                plan.set_positions(None)
            if stats:
                st = plan.stats(sp)
        else:
            if max_iterations is None:  # a monotone Pablo loop settles within n iterations
                max_iterations = 4 * max(inp.lengths + [0]) + 64
            lay = N.Layout(inp.kind, inp.n, _i64(inp.offsets), _i64(inp.lengths), inp.basis_stride,
                           _i64(offs), stride)
            N.check(N.lib().bg_interp_run(self._interp, C.byref(lay), inp.data.data_ptr(),
                                          out_ptr or None, cnt_ptr or None, max_iterations, sp),
                    "bg_interp_run")
        return ScanResult(out if streams else None, cnt, offs, words, pos, st)

    def close(self):
        for p in self._plans.values():
            p.close()
        self._plans.clear()
        if self._handle:
            N.lib().bg_program_destroy(self._handle)
            self._handle = None
        if self._interp:
            N.lib().bg_interp_destroy(self._interp)
            self._interp = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def transpose(bytestream: torch.Tensor, bitstream: torch.Tensor, stream=None):
    """Byte -> basis transpose into a caller-allocated tensor (reference shapes
    ``uint8 [S, M, Npad]`` -> ``uint32 [S, M, 8, Npad/32]``)."""
    if bytestream.dtype != torch.uint8 or bitstream.dtype not in (torch.uint32, torch.int32):
        raise TypeError("transpose expects uint8 bytes and uint32 planes")
    if not (bytestream.is_cuda and bitstream.is_cuda):
        raise ValueError("transpose expects CUDA tensors")
    if not bytestream.is_contiguous() or not bitstream.is_contiguous():
        raise ValueError("transpose expects contiguous tensors")
    npad = bytestream.shape[-1]
    m = bytestream.numel() // max(1, npad)
    if npad % 32 or bitstream.shape[-2:] != (8, npad // 32) or bitstream.numel() != m * npad // 4:
        raise ValueError(f"shape mismatch: {tuple(bytestream.shape)} -> {tuple(bitstream.shape)}")
    N.check(N.lib().bg_transpose(bytestream.data_ptr(), bitstream.data_ptr(), npad, m,
                                 _stream_ptr(stream)), "bg_transpose")
