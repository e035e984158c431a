/* bitgen_gb300 runtime: the C ABI declared in include/bitgen_gb300.h.
 *
 * Host side of the engine: NVRTC compilation of generated scan kernels for sm_103a (with an
 * on-disk cubin cache), per-layout launch plans holding the device-side tables and look-back
 * records, the stand-alone byte -> basis transpose kernel, and a whole-stream executor for
 * Pablo programs that keep while/if blocks.  It replaces the reference's cuda-python driver
 * (bitgen/backend/cuda/cuda_kernel.py) and its torch extension (bitgen/template/cuda/).
 */
#include <cuda_runtime.h>
#include <nvJitLink.h>
#include <nvrtc.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/bitgen_gb300.h"
#include "bg_params.h"
#include "bg_transpose.cuh"

extern "C" const char *bg_embedded_device_cuh;
extern "C" const char *bg_embedded_params_h;
extern "C" const char *bg_embedded_transpose_cuh;

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string &msg) {
  g_last_error = msg;
  return code;
}

#define BG_CUDA(call)                                                                 \
  do {                                                                                \
    cudaError_t e_ = (call);                                                          \
    if (e_ != cudaSuccess)                                                            \
      return fail(BG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));  \
  } while (0)

bool aligned16(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

/* ------------------------------------------------------------------------------------ */
/* Stand-alone transpose: one thread per 32-byte word, grid-stride, coalesced stores.     */
/* ------------------------------------------------------------------------------------ */
__global__ void __launch_bounds__(256) bg_transpose_kernel(const uint8_t *__restrict__ bytes,
                                                           uint32_t *__restrict__ basis,
                                                           int64_t W, int64_t total) {
  for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < total;
       g += (int64_t)gridDim.x * blockDim.x) {
    const int64_t input = g / W, w = g - input * W;
    const uint4 *q = reinterpret_cast<const uint4 *>(bytes + 32 * g);
    const uint4 a = __ldg(q), c = __ldg(q + 1);
    const uint32_t u[8] = {a.x, a.y, a.z, a.w, c.x, c.y, c.z, c.w};
    uint32_t o[8];
    bg::transpose32(u, o);
    uint32_t *dst = basis + input * 8 * W + w;
#pragma unroll
    for (int i = 0; i < 8; ++i) dst[i * W] = o[i];
  }
}

__global__ void bg_prologue_kernel(uint32_t *state) {
  state[0] = 0u;
  state[6] = 0u; /* match positions written */
  state[7] = 0u;
  unsigned long long *ep = reinterpret_cast<unsigned long long *>(state + 2);
  *ep = *ep + 1ull;
}

/* Carry scan of the pre-pass additions.  Block k handles addition k, whose bitmaps (see
 * bg_device.cuh, pre_rows) hold for every row of 32 tiles the tiles that generate (G) and
 * propagate (P) a carry.  Bit l of A = G | P and B = G belong to tile l of the row, so
 * A + B + carry-in gives the carry entering every tile of the row at once: bit l of
 * (A + B + c) ^ A ^ B, and bit 32 of the sum leaves the row.  The last tile of each input gets
 * A = B = 0: its carry-out only enters the next input's first tile, which must see zero.  Each
 * thread folds a contiguous run of rows into (carry-out for carry-in 0, for carry-in 1), the
 * folds are scanned across the block, and a second walk writes the carry-in bitmap. */
__device__ __forceinline__ uint32_t row_kill(int64_t row, const int64_t *tile_prefix, int n_inputs,
                                             int &in) {
  /* inputs whose last tile lies in this row (the cursor only moves forward) */
  uint32_t kill = 0u;
  const int64_t lo = row * 32, hi = lo + 32;
  while (in < n_inputs && tile_prefix[in + 1] <= hi) {
    const int64_t last = tile_prefix[in + 1] - 1;
    if (last >= lo) kill |= 1u << (last - lo);
    ++in;
  }
  return kill;
}

__device__ __forceinline__ void carry_scan_block(int k, uint32_t *pre_bits, int64_t n_tiles,
                                                 const int64_t *tile_prefix, int n_inputs) {
  __shared__ uint32_t wg[32], wp[32];
  const int64_t R = (n_tiles + 31) / 32;
  const uint32_t *Gw = pre_bits + 3 * R * k, *Pw = Gw + R;
  uint32_t *Cw = pre_bits + 3 * R * k + 2 * R;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
  const int64_t per = (R + blockDim.x - 1) / blockDim.x;
  const int64_t r0 = (int64_t)tid * per < R ? (int64_t)tid * per : R;
  const int64_t r1 = r0 + per < R ? r0 + per : R;
  int in0 = 0;
  {
    int a = 0, b = n_inputs; /* input containing tile 32 * r0 */
    while (b - a > 1) {
      const int m = (a + b) >> 1;
      if (tile_prefix[m] <= r0 * 32) a = m; else b = m;
    }
    in0 = a;
  }
  /* rows are taken RB at a time, their bitmap words loaded together (the loads of a thread's
   * rows do not wait for one another; only the carry chains through them) */
  constexpr int RB = 8;
  uint32_t c0 = 0u, c1 = 1u;
  int in = in0;
  for (int64_t rb = r0; rb < r1; rb += RB) {
    uint32_t g[RB], q[RB];
#pragma unroll
    for (int i = 0; i < RB; ++i) {
      g[i] = rb + i < r1 ? Gw[rb + i] : 0u;
      q[i] = rb + i < r1 ? Pw[rb + i] : 0u;
    }
#pragma unroll
    for (int i = 0; i < RB; ++i) {
      if (rb + i >= r1) break;
      const uint32_t kill = row_kill(rb + i, tile_prefix, n_inputs, in);
      const uint32_t A = (g[i] | q[i]) & ~kill, B = g[i] & ~kill;
      c0 = (uint32_t)((((unsigned long long)A + B + c0) >> 32) & 1ull);
      c1 = (uint32_t)((((unsigned long long)A + B + c1) >> 32) & 1ull);
    }
  }
  /* (G, P) of this thread's run: carry-out = G | (P & carry-in) */
  uint32_t iG = c0, iP = c1 & ~c0 & 1u;
  for (int d = 1; d < 32; d <<= 1) {
    const uint32_t uG = __shfl_up_sync(0xffffffffu, iG, d), uP = __shfl_up_sync(0xffffffffu, iP, d);
    if (lane >= d) {
      iG = iG | (iP & uG);
      iP &= uP;
    }
  }
  if (lane == 31) {
    wg[warp] = iG;
    wp[warp] = iP;
  }
  __syncthreads();
  if (warp == 0) {
    uint32_t a = lane < nwarps ? wg[lane] : 0u;
    uint32_t b = lane < nwarps ? wp[lane] : 1u;
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t uG = __shfl_up_sync(0xffffffffu, a, d), uP = __shfl_up_sync(0xffffffffu, b, d);
      if (lane >= d) {
        a = a | (b & uG);
        b &= uP;
      }
    }
    wg[lane] = a;
    wp[lane] = b;
  }
  __syncthreads();
  /* carry entering this thread's first row: the exclusive prefix (carry-in 0 at tile 0) */
  uint32_t eG = __shfl_up_sync(0xffffffffu, iG, 1), eP = __shfl_up_sync(0xffffffffu, iP, 1);
  if (lane == 0) {
    eG = 0u;
    eP = 1u;
  }
  uint32_t c = eG;
  if (warp > 0) c = eG | (eP & wg[warp - 1]);
  in = in0;
  for (int64_t rb = r0; rb < r1; rb += RB) {
    uint32_t g[RB], q[RB];
#pragma unroll
    for (int i = 0; i < RB; ++i) {
      g[i] = rb + i < r1 ? Gw[rb + i] : 0u;
      q[i] = rb + i < r1 ? Pw[rb + i] : 0u;
    }
#pragma unroll
    for (int i = 0; i < RB; ++i) {
      if (rb + i >= r1) break;
      const uint32_t kill = row_kill(rb + i, tile_prefix, n_inputs, in);
      const uint32_t A = (g[i] | q[i]) & ~kill, B = g[i] & ~kill;
      const unsigned long long sum = (unsigned long long)A + B + c;
      Cw[rb + i] = (uint32_t)sum ^ A ^ B;
      c = (uint32_t)((sum >> 32) & 1ull);
    }
  }
}

__global__ void __launch_bounds__(1024) bg_carry_scan_kernel(uint32_t *pre_bits, int64_t n_tiles,
                                                             const int64_t *tile_prefix,
                                                             int n_inputs) {
  carry_scan_block(blockIdx.x, pre_bits, n_tiles, tile_prefix, n_inputs);
}

/* Work list of the split form's execute pass: the (part, tile row) pairs where the part has
 * something to run, a row being 32 consecutive tiles.  The classify pass leaves, for every row
 * and run-mask word, the OR of the row's 32 masks (`rowrun`, [n_run][rows]); part p has work in
 * a row when one of its (word, mask) pairs (`pmask`) meets it.  Block p lists part p's rows in
 * increasing order at work + H + n_parts + p * rows and stores their count at work[H + p]
 * (H = BG_WORK_HEAD; block 0 also zeroes the execute pass's claim counters, work[0, H)):
 * each warp takes a contiguous block of rows, 32 rows per step (one per lane, coalesced loads,
 * a ballot to keep them in order), and the warps' counts are scanned across the block.  The
 * execute pass orders the parts one after the other (part-major, so that the whole GPU runs one
 * part at a time) and claims a part's rows in increasing order. */
constexpr int64_t LIST_KEEP = 1024; /* steps whose ballots a block keeps in shared memory */
__device__ __forceinline__ void work_list_block(int p, const uint32_t *rowrun,
                                                const uint32_t *pmask, int pmw, uint32_t *work,
                                                int n_parts, int64_t rows) {
  __shared__ uint32_t wsum[32];
  __shared__ uint32_t bal[LIST_KEEP];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const uint32_t *pm = pmask + (int64_t)p * pmw * 2;
  uint32_t *out = work + BG_WORK_HEAD + n_parts + (int64_t)p * rows;
  if (p == 0)
    for (int i = threadIdx.x; i < BG_WORK_HEAD; i += blockDim.x) work[i] = 0u;
  const int64_t steps = (rows + 31) / 32;
  const int64_t per = (steps + nwarps - 1) / nwarps;
  const int64_t s0 = (int64_t)warp * per < steps ? (int64_t)warp * per : steps;
  const int64_t s1 = s0 + per < steps ? s0 + per : steps;
  /* the part's (word, mask) pairs, in registers for up to PM pairs */
  constexpr int PM = 4;
  uint32_t pw_[PM], pm_[PM];
#pragma unroll
  for (int e = 0; e < PM; ++e) {
    pw_[e] = e < pmw ? pm[2 * e] : 0u;
    pm_[e] = e < pmw ? pm[2 * e + 1] : 0u;
  }
  auto present_any = [&](int64_t step) -> uint32_t {
    const int64_t r = step * 32 + lane;
    uint32_t any = 0u;
    if (step < s1 && r < rows) {
      if (pmw <= PM) {
#pragma unroll
        for (int e = 0; e < PM; ++e)
          if (pm_[e]) any |= rowrun[(int64_t)pw_[e] * rows + r] & pm_[e];
      } else {
        for (int e = 0; e < pmw; ++e) {
          const uint32_t m = pm[2 * e + 1];
          if (m) any |= rowrun[(int64_t)pm[2 * e] * rows + r] & m;
        }
      }
    }
    return any;
  };
  /* first walk: SB steps at a time, their loads issued together; the ballots are kept */
  constexpr int SB = 8;
  const bool keep = steps <= LIST_KEEP;
  uint32_t cnt = 0;
  for (int64_t sb = s0; sb < s1; sb += SB) {
    uint32_t any[SB];
#pragma unroll
    for (int i = 0; i < SB; ++i) any[i] = present_any(sb + i);
#pragma unroll
    for (int i = 0; i < SB; ++i) {
      if (sb + i >= s1) break;
      const uint32_t b = __ballot_sync(0xffffffffu, any[i] != 0u);
      cnt += __popc(b);
      if (keep && lane == 0) bal[sb + i] = b;
    }
  }
  if (lane == 0) wsum[warp] = cnt;
  __syncthreads();
  uint32_t pos = 0, total = 0;
  for (int w = 0; w < nwarps; ++w) {
    if (w < warp) pos += wsum[w];
    total += wsum[w];
  }
  for (int64_t st = s0; st < s1; ++st) {
    const uint32_t b = keep ? bal[st] : __ballot_sync(0xffffffffu, present_any(st) != 0u);
    if ((b >> lane) & 1u) out[pos + __popc(b & ((1u << lane) - 1u))] = (uint32_t)(st * 32 + lane);
    pos += __popc(b);
  }
  if (threadIdx.x == 0) work[BG_WORK_HEAD + p] = total;
}

/* work_list_block for launches of at most WARP_LIST_ROWS rows: one warp lists part p, walking
 * the rows 32 at a time (no block-wide scan), so one block serves a part per warp. */
constexpr int64_t WARP_LIST_ROWS = 256;
__device__ __forceinline__ void work_list_warp(int p, const uint32_t *rowrun, const uint32_t *pmask,
                                               int pmw, uint32_t *work, int n_parts, int64_t rows) {
  const int lane = threadIdx.x & 31;
  const uint32_t *pm = pmask + (int64_t)p * pmw * 2;
  uint32_t *out = work + BG_WORK_HEAD + n_parts + (int64_t)p * rows;
  if (p == 0)
    for (int i = lane; i < BG_WORK_HEAD; i += 32) work[i] = 0u;
  uint32_t pos = 0;
  for (int64_t st = 0; st * 32 < rows; ++st) {
    const int64_t r = st * 32 + lane;
    uint32_t any = 0u;
    if (r < rows)
      for (int e = 0; e < pmw; ++e) {
        const uint32_t m = pm[2 * e + 1];
        if (m) any |= rowrun[(int64_t)pm[2 * e] * rows + r] & m;
      }
    const uint32_t b = __ballot_sync(0xffffffffu, any != 0u);
    if ((b >> lane) & 1u) out[pos + __popc(b & ((1u << lane) - 1u))] = (uint32_t)r;
    pos += __popc(b);
  }
  if (lane == 0) work[BG_WORK_HEAD + p] = pos;
}

/* The split form's row-level work between classify and execute in one launch: blocks
 * [0, n_pre) scan the pre-pass carries (one addition each), the other blocks list the parts'
 * rows: one part per block, or, for launches of few rows, one part per warp. */
__global__ void __launch_bounds__(512, 2) bg_rows_kernel(uint32_t *pre_bits, int64_t n_tiles,
                                                       const int64_t *tile_prefix, int n_inputs,
                                                       int n_pre, const uint32_t *rowrun,
                                                       const uint32_t *pmask, int pmw,
                                                       uint32_t *work, int n_parts, int64_t rows) {
  asm volatile("griddepcontrol.wait;" ::: "memory"); /* classify's results */
  if ((int)blockIdx.x < n_pre) {
    carry_scan_block(blockIdx.x, pre_bits, n_tiles, tile_prefix, n_inputs);
  } else if (rows <= WARP_LIST_ROWS) {
    const int p = ((int)blockIdx.x - n_pre) * (int)(blockDim.x >> 5) + (int)(threadIdx.x >> 5);
    if (p < n_parts) work_list_warp(p, rowrun, pmask, pmw, work, n_parts, rows);
  } else {
    work_list_block(blockIdx.x - n_pre, rowrun, pmask, pmw, work, n_parts, rows);
  }
}

/* 32-bit words of the split form's work list (claim counters, counts, rows per part, row
 * summaries). */
int64_t work_words(const bg_kernel_desc &d, int64_t tiles) {
  const int64_t rows = (tiles + 31) / 32;
  return d.n_run > 0 ? BG_WORK_HEAD + (int64_t)d.n_parts * (1 + rows) + (int64_t)d.n_run * rows
                    : 0;
}

/* 64-bit words of a records buffer for `tiles` tiles: one look-back record per addition and
 * tile, then the pre-pass bitmaps (3 words of 32 tiles per pre-pass addition). */
int64_t record_words(const bg_kernel_desc &d, int64_t tiles) {
  const int64_t rows = (tiles + 31) / 32;
  return (int64_t)std::max(1, d.n_adds) * tiles + (3 * (int64_t)d.n_pre * rows + 1) / 2;
}

int sm_count() {
  static int n = -1;
  if (n < 0) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
      n = 1;
  }
  return n;
}

/* FNV-1a 64 */
uint64_t fnv(const std::string &s, uint64_t h = 1469598103934665603ull) {
  for (unsigned char c : s) {
    h ^= c;
    h *= 1099511628211ull;
  }
  return h;
}

}  // namespace

/* ======================================================================================== */
/* Program                                                                                  */
/* ======================================================================================== */
struct bg_program {
  bg_kernel_desc desc{};
  std::string name;
  std::string log;
  std::vector<char> cubin;
  cudaLibrary_t lib = nullptr;
  cudaKernel_t kernel = nullptr;
  cudaKernel_t pre_kernel = nullptr; /* carry pre-pass, when desc.n_pre > 0 (single form) */
  cudaKernel_t cls_kernel = nullptr; /* classify pass of the split form (desc.n_run > 0)  */
  const uint32_t *pmask = nullptr;   /* split form: per part, pmw (word, mask) pairs        */
  int pmw = 0;
  int regs = 0, local_bytes = 0, blocks_per_sm = 1, pre_blocks_per_sm = 1;
  int cls_block = 0, cls_smem = 0; /* classify launch (bg_cls_cfg of the program)          */
};

struct bg_plan {
  bg_program *prog = nullptr;
  bg_layout layout{};
  int64_t n_tiles = 0;
  int64_t *d_tables = nullptr; /* in_off | in_len | tile_prefix | out_off */
  unsigned long long *d_records = nullptr;
  uint32_t *d_state = nullptr;
  uint32_t *d_runs = nullptr; /* split form: [n_run][cap_tiles] run masks */
  uint32_t *d_work = nullptr; /* split form: work list */
  int grid = 1;
  int64_t debug_wait_tile = -1;
  int64_t spin_limit = 0;
  int64_t cap_inputs = 0, cap_tiles = 0;
  unsigned long long *positions = nullptr;
  int64_t pos_capacity = 0;
  unsigned long long *d_set = nullptr; /* position set of launches without output streams */
  int64_t set_slots = 0;
  bool count_only = false;             /* a set sized for counting, no positions written  */
  int64_t *h_stage = nullptr; /* pinned staging of the tables */
  cudaEvent_t staged = nullptr;
  bool staged_pending = false;
};

extern "C" {

const char *bg_status_string(int s) {
  switch (s) {
    case BG_OK: return "ok";
    case BG_ERR_INVALID: return "invalid argument";
    case BG_ERR_CUDA: return "CUDA error";
    case BG_ERR_COMPILE: return "NVRTC compilation failed";
    case BG_ERR_TIMEOUT: return "bounded device wait timed out";
    case BG_ERR_ALIGN: return "input not 16-byte aligned";
    case BG_ERR_NOMEM: return "out of memory";
    case BG_ERR_DEVICE: return "device reported an internal inconsistency";
    case BG_ERR_CAPACITY: return "output buffer too small";
    default: return "unknown status";
  }
}

const char *bg_last_error(void) { return g_last_error.c_str(); }

int bg_interp_fail(int code, const char *msg) { return fail(code, msg ? msg : ""); }

int bg_device_available(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n > 0 ? 1 : 0;
}

int bg_transpose(const uint8_t *bytes, uint32_t *basis, int64_t n_bytes_padded, int64_t n_inputs,
                 void *stream) {
  if (!bytes || !basis || n_bytes_padded < 0 || n_inputs < 0 || n_bytes_padded % 32)
    return fail(BG_ERR_INVALID, "bg_transpose: bad arguments");
  if (!aligned16(bytes)) return fail(BG_ERR_ALIGN, "bg_transpose: bytes not 16-byte aligned");
  const int64_t W = n_bytes_padded / 32, total = W * n_inputs;
  if (total == 0) return BG_OK;
  const int64_t want = (total + 255) / 256;
  const int grid = (int)std::min<int64_t>(want, (int64_t)sm_count() * 16);
  bg_transpose_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(bytes, basis, W, total);
  BG_CUDA(cudaGetLastError());
  return BG_OK;
}

/* One NVRTC compilation of `src` to a cubin (relocatable when `rdc`). */
static int nvrtc_one(const std::string &src, const std::string &name, bool rdc, std::string &log,
                     std::vector<char> &cubin) {
  /* "//@@BG_MAXREG n" in the source caps registers in every translation unit (the linker
   * requires callees of a __launch_bounds__ kernel to fit its register budget); a unit whose
   * kernel calls only functions of its own unit may set its own cap with "//@@BG_UNITREG n" */
  std::string maxreg;
  const size_t up = src.find("//@@BG_UNITREG ");
  const size_t mp = src.find("//@@BG_MAXREG ");
  if (up != std::string::npos)
    maxreg = "--maxrregcount=" + std::to_string(atoi(src.c_str() + up + 15));
  else if (mp != std::string::npos)
    maxreg = "--maxrregcount=" + std::to_string(atoi(src.c_str() + mp + 14));
  std::vector<const char *> base = {"--gpu-architecture=sm_103a", "-std=c++17", "-lineinfo",
                                    "--device-as-default-execution-space"};
  if (rdc) base.push_back("--relocatable-device-code=true");
  if (!maxreg.empty()) base.push_back(maxreg.c_str());
  const int n_opts = (int)base.size();
  nvrtcProgram prog;
  const char *headers[] = {bg_embedded_device_cuh, bg_embedded_params_h, bg_embedded_transpose_cuh};
  const char *names[] = {"bg_device.cuh", "bg_params.h", "bg_transpose.cuh"};
  if (nvrtcCreateProgram(&prog, src.c_str(), (name + ".cu").c_str(), 3, headers, names) !=
      NVRTC_SUCCESS)
    return fail(BG_ERR_COMPILE, "nvrtcCreateProgram failed");
  nvrtcResult r = nvrtcCompileProgram(prog, n_opts, base.data());
  size_t logsz = 0;
  nvrtcGetProgramLogSize(prog, &logsz);
  log.assign(logsz, '\0');
  if (logsz) nvrtcGetProgramLog(prog, &log[0]);
  if (r != NVRTC_SUCCESS) {
    nvrtcDestroyProgram(&prog);
    return fail(BG_ERR_COMPILE, std::string("NVRTC: ") + nvrtcGetErrorString(r) + "\n" + log);
  }
  size_t sz = 0;
  nvrtcGetCUBINSize(prog, &sz);
  cubin.resize(sz);
  nvrtcGetCUBIN(prog, cubin.data());
  nvrtcDestroyProgram(&prog);
  return BG_OK;
}

/* Sources generated with "//@@BG_PART" / "//@@BG_KERNEL" section markers are compiled as one
 * relocatable translation unit per section (prelude + section) on parallel host threads and
 * linked with nvJitLink; other sources are compiled whole. */
static int compile_sections(const std::string &src, const std::string &name, std::string &log,
                            std::vector<char> &cubin) {
  const std::string PART = "//@@BG_PART\n", KERN = "//@@BG_KERNEL\n";
  std::vector<size_t> cuts;
  for (size_t pos = src.find("//@@BG_"); pos != std::string::npos; pos = src.find("//@@BG_", pos + 1))
    if (src.compare(pos, PART.size(), PART) == 0 || src.compare(pos, KERN.size(), KERN) == 0)
      cuts.push_back(pos);
  if (cuts.size() < 3) return nvrtc_one(src, name, false, log, cubin);
  const std::string prelude = src.substr(0, cuts[0]);
  std::vector<std::string> units;
  for (size_t i = 0; i < cuts.size(); ++i) {
    const size_t e = i + 1 < cuts.size() ? cuts[i + 1] : src.size();
    units.push_back(prelude + src.substr(cuts[i], e - cuts[i]));
  }
  const size_t n = units.size();
  std::vector<std::vector<char>> objs(n);
  std::vector<std::string> logs(n), errs(n);
  std::vector<int> rcs(n, BG_OK);
  unsigned hw = std::thread::hardware_concurrency();
  const size_t workers = std::max<size_t>(1, std::min<size_t>(n, hw ? hw : 4));
  std::vector<std::thread> pool;
  std::atomic<size_t> next{0};
  for (size_t w = 0; w < workers; ++w)
    pool.emplace_back([&]() {
      for (size_t i = next++; i < n; i = next++) {
        rcs[i] = nvrtc_one(units[i], name + "_" + std::to_string(i), true, logs[i], objs[i]);
        if (rcs[i] != BG_OK) errs[i] = g_last_error;
      }
    });
  for (auto &t : pool) t.join();
  for (size_t i = 0; i < n; ++i) {
    if (!logs[i].empty()) log += logs[i];
    if (rcs[i] != BG_OK) return fail(rcs[i], errs[i]);
  }
  nvJitLinkHandle h;
  const char *lopts[] = {"-arch=sm_103a"};
  if (nvJitLinkCreate(&h, 1, lopts) != NVJITLINK_SUCCESS)
    return fail(BG_ERR_COMPILE, "nvJitLinkCreate failed");
  int rc = BG_OK;
  for (size_t i = 0; i < n && rc == BG_OK; ++i) {
    const std::string nm = name + "_" + std::to_string(i) + ".cubin";
    if (nvJitLinkAddData(h, NVJITLINK_INPUT_CUBIN, objs[i].data(), objs[i].size(), nm.c_str()) !=
        NVJITLINK_SUCCESS)
      rc = BG_ERR_COMPILE;
  }
  if (rc == BG_OK && nvJitLinkComplete(h) != NVJITLINK_SUCCESS) rc = BG_ERR_COMPILE;
  if (rc != BG_OK) {
    size_t ls = 0;
    nvJitLinkGetErrorLogSize(h, &ls);
    std::string el(ls, '\0');
    if (ls) nvJitLinkGetErrorLog(h, &el[0]);
    nvJitLinkDestroy(&h);
    return fail(BG_ERR_COMPILE, "nvJitLink: " + el);
  }
  size_t sz = 0;
  nvJitLinkGetLinkedCubinSize(h, &sz);
  cubin.resize(sz);
  nvJitLinkGetLinkedCubin(h, cubin.data());
  nvJitLinkDestroy(&h);
  return BG_OK;
}

static int compile_cubin(const std::string &src, const std::string &name, std::string &log,
                         std::vector<char> &cubin) {
  int major = 0, minor = 0;
  nvrtcVersion(&major, &minor);
  std::string key = src + "|" + name + "|" + std::to_string(major) + "." + std::to_string(minor);
  key += "|sm_103a|rdc-sections-v1";
  key += bg_embedded_device_cuh;
  key += bg_embedded_params_h;
  key += bg_embedded_transpose_cuh;
  char hex[40];
  snprintf(hex, sizeof hex, "%016llx%016llx", (unsigned long long)fnv(key),
           (unsigned long long)fnv(key, 0x84222325cbf29ce4ull));
  const char *dir = getenv("BG_CACHE_DIR");
  std::string path = dir && *dir ? std::string(dir) + "/" + hex + ".cubin" : std::string();
  if (!path.empty()) {
    if (FILE *f = fopen(path.c_str(), "rb")) {
      fseek(f, 0, SEEK_END);
      long sz = ftell(f);
      fseek(f, 0, SEEK_SET);
      cubin.resize(sz > 0 ? (size_t)sz : 0);
      size_t got = sz > 0 ? fread(cubin.data(), 1, (size_t)sz, f) : 0;
      fclose(f);
      if (sz > 0 && got == (size_t)sz) {
        log = "cubin cache hit " + path;
        return BG_OK;
      }
      cubin.clear();
    }
  }
  const int rc = compile_sections(src, name, log, cubin);
  if (rc != BG_OK) return rc;
  if (!path.empty()) {
    std::string tmp = path + ".tmp" + std::to_string((long long)getpid());
    if (FILE *f = fopen(tmp.c_str(), "wb")) {
      fwrite(cubin.data(), 1, cubin.size(), f);
      fclose(f);
      rename(tmp.c_str(), path.c_str());
    }
  }
  return BG_OK;
}

int bg_nvrtc_check(const char *source, size_t source_len, const char *name, char *log_buf,
                   size_t log_len) {
  if (!source || !name) return fail(BG_ERR_INVALID, "bg_nvrtc_check: bad arguments");
  std::string src(source, source_len ? source_len : strlen(source)), log;
  std::vector<char> cubin;
  const int rc = compile_cubin(src, name, log, cubin);
  if (log_buf && log_len) {
    const std::string &m = rc == BG_OK ? log : g_last_error;
    size_t n = std::min(log_len - 1, m.size());
    memcpy(log_buf, m.data(), n);
    log_buf[n] = '\0';
  }
  return rc;
}

int bg_program_create(const bg_kernel_desc *desc, bg_program **out) {
  if (!desc || !out || !desc->source || !desc->name || desc->wpt < 1 || desc->wpt > 8 ||
      desc->halo_lanes < 0 || desc->tail_lanes < 0 || desc->halo_lanes + desc->tail_lanes > 31 ||
      desc->n_outputs < 0 || desc->n_adds < 0 || desc->n_pre < 0 || desc->n_pre > desc->n_adds ||
      desc->n_run < 0 ||
      desc->block < 32 || desc->block % 32)
    return fail(BG_ERR_INVALID, "bg_program_create: bad descriptor");
  *out = nullptr;
  bg_program *p = new (std::nothrow) bg_program();
  if (!p) return fail(BG_ERR_NOMEM, "bg_program_create: out of host memory");
  p->desc = *desc;
  p->name = desc->name;
  p->desc.name = p->name.c_str();
  p->desc.source = nullptr;
  std::string src(desc->source, desc->source_len ? desc->source_len : strlen(desc->source));
  int rc = compile_cubin(src, p->name, p->log, p->cubin);
  if (rc != BG_OK) {
    std::string keep = g_last_error;
    delete p;
    g_last_error = keep;
    return rc;
  }
  cudaError_t e = cudaLibraryLoadData(&p->lib, p->cubin.data(), nullptr, nullptr, 0, nullptr,
                                      nullptr, 0);
  if (e == cudaSuccess) e = cudaLibraryGetKernel(&p->kernel, p->lib, p->name.c_str());
  if (e == cudaSuccess && desc->n_run > 0) {
    e = cudaLibraryGetKernel(&p->cls_kernel, p->lib, (p->name + "_cls").c_str());
    void *pm = nullptr;
    size_t pm_bytes = 0;
    if (e == cudaSuccess) e = cudaLibraryGetGlobal(&pm, &pm_bytes, p->lib, "bg_pmask");
    if (e == cudaSuccess) {
      p->pmask = static_cast<const uint32_t *>(pm);
      p->pmw = (int)(pm_bytes / (sizeof(uint32_t) * 2 * (size_t)std::max(1, desc->n_parts)));
    }
    /* classify's block size and dynamic shared memory; programs without the table use the
     * program's block and static shared memory */
    void *cfg = nullptr;
    size_t cfg_bytes = 0;
    p->cls_block = desc->block;
    if (e == cudaSuccess &&
        cudaLibraryGetGlobal(&cfg, &cfg_bytes, p->lib, "bg_cls_cfg") == cudaSuccess &&
        cfg_bytes >= 2 * sizeof(uint32_t)) {
      uint32_t c[2] = {0, 0};
      e = cudaMemcpy(c, cfg, sizeof c, cudaMemcpyDeviceToHost);
      if (e == cudaSuccess && (c[0] == 0 || c[0] > 1024 || c[0] % 32 != 0 || c[1] > 227u * 1024u))
        e = cudaErrorInvalidValue;
      if (e == cudaSuccess) {
        p->cls_block = (int)c[0];
        p->cls_smem = (int)c[1];
        e = cudaFuncSetAttribute((const void *)p->cls_kernel,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, p->cls_smem);
      }
    } else {
      cudaGetLastError();
    }
  }
  else if (e == cudaSuccess && desc->n_pre > 0)
    e = cudaLibraryGetKernel(&p->pre_kernel, p->lib, (p->name + "_pre").c_str());
  if (e != cudaSuccess) {
    std::string msg = std::string("loading the compiled program: ") + cudaGetErrorString(e);
    if (p->lib) cudaLibraryUnload(p->lib);
    delete p;
    return fail(BG_ERR_CUDA, msg);
  }
  cudaFuncAttributes attr{};
  if (cudaFuncGetAttributes(&attr, (const void *)p->kernel) == cudaSuccess) {
    p->regs = attr.numRegs;
    p->local_bytes = (int)attr.localSizeBytes;
  } else {
    cudaGetLastError();
  }
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, (const void *)p->kernel, desc->block,
                                                    0) == cudaSuccess && nb > 0) {
    p->blocks_per_sm = nb;
  } else {
    cudaGetLastError();
    int regs = p->regs > 0 ? p->regs : 128;
    p->blocks_per_sm = std::max(1, 65536 / (regs * desc->block));
  }
  if (p->pre_kernel || p->cls_kernel) {
    nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &nb, (const void *)(p->cls_kernel ? p->cls_kernel : p->pre_kernel),
            p->cls_kernel ? p->cls_block : desc->block, p->cls_kernel ? (size_t)p->cls_smem : 0) ==
            cudaSuccess && nb > 0)
      p->pre_blocks_per_sm = nb;
    else
      cudaGetLastError();
  }
  *out = p;
  return BG_OK;
}

int bg_program_log(const bg_program *prog, char *buf, size_t len) {
  if (!prog || !buf || !len) return fail(BG_ERR_INVALID, "bg_program_log: bad arguments");
  size_t n = std::min(len - 1, prog->log.size());
  memcpy(buf, prog->log.data(), n);
  buf[n] = '\0';
  return BG_OK;
}

int bg_program_info(const bg_program *prog, int32_t *regs, int32_t *local_bytes,
                    int32_t *max_blocks_per_sm) {
  if (!prog) return fail(BG_ERR_INVALID, "bg_program_info: null program");
  if (regs) *regs = prog->regs;
  if (local_bytes) *local_bytes = prog->local_bytes;
  if (max_blocks_per_sm) *max_blocks_per_sm = prog->blocks_per_sm;
  return BG_OK;
}

int bg_program_destroy(bg_program *prog) {
  if (!prog) return BG_OK;
  if (prog->lib) cudaLibraryUnload(prog->lib);
  delete prog;
  return BG_OK;
}

/* ======================================================================================== */
/* Plans                                                                                    */
/* ======================================================================================== */
/* tables for a layout: in_off | in_len | tile_prefix | out_off; returns the tile count or < 0 */
static int64_t build_tables(const bg_program *prog, const bg_layout *L, int64_t *t) {
  const int64_t n = L->n_inputs;
  const int64_t tile_words =
      (int64_t)(32 - prog->desc.halo_lanes - prog->desc.tail_lanes) * prog->desc.wpt;
  int64_t *in_off = t, *in_len = t + n, *prefix = t + 2 * n, *out_off = t + 3 * n + 1;
  prefix[0] = 0;
  for (int64_t i = 0; i < n; ++i) {
    if (L->in_len[i] < 0 || L->in_off[i] < 0) return -fail(BG_ERR_INVALID, "layout: negative offset or length");
    if (L->input_kind == BG_INPUT_BYTES && (L->in_off[i] & 15))
      return -fail(BG_ERR_ALIGN, "layout: byte offsets must be multiples of 16");
    in_off[i] = L->in_off[i];
    in_len[i] = L->in_len[i];
    out_off[i] = L->out_off[i];
    const int64_t W = (L->in_len[i] + 31) / 32;
    prefix[i + 1] = prefix[i] + std::max<int64_t>(1, (W + tile_words - 1) / tile_words);
  }
  return prefix[n];
}

static bool layout_ok(const bg_layout *L) {
  return L && L->n_inputs >= 1 && L->in_off && L->in_len && L->out_off &&
         (L->input_kind == BG_INPUT_BYTES || L->input_kind == BG_INPUT_BASIS);
}

int bg_plan_reserve(bg_program *prog, int32_t input_kind, int32_t max_inputs, int64_t max_tiles,
                    bg_plan **out) {
  if (!prog || !out || max_inputs < 1 || max_tiles < 1 || max_tiles >= (int64_t)0xffffffffll ||
      (input_kind != BG_INPUT_BYTES && input_kind != BG_INPUT_BASIS))
    return fail(BG_ERR_INVALID, "bg_plan_reserve: bad arguments");
  *out = nullptr;
  bg_plan *p = new (std::nothrow) bg_plan();
  if (!p) return fail(BG_ERR_NOMEM, "bg_plan_reserve: out of host memory");
  p->prog = prog;
  p->layout.input_kind = input_kind;
  p->cap_inputs = max_inputs;
  p->cap_tiles = max_tiles;
  auto cleanup = [&](int code, const std::string &m) {
    bg_plan_destroy(p);
    return fail(code, m);
  };
  const size_t ntab = 4 * (size_t)max_inputs + 1;
  if (cudaMalloc(&p->d_tables, ntab * sizeof(int64_t)) != cudaSuccess)
    return cleanup(BG_ERR_NOMEM, "bg_plan_reserve: tables");
  if (cudaMallocHost(&p->h_stage, ntab * sizeof(int64_t)) != cudaSuccess)
    return cleanup(BG_ERR_NOMEM, "bg_plan_reserve: staging");
  if (cudaEventCreateWithFlags(&p->staged, cudaEventDisableTiming) != cudaSuccess)
    return cleanup(BG_ERR_CUDA, "bg_plan_reserve: event");
  const size_t nrec = (size_t)record_words(prog->desc, max_tiles);
  if (cudaMalloc(&p->d_records, nrec * sizeof(unsigned long long)) != cudaSuccess)
    return cleanup(BG_ERR_NOMEM, "bg_plan_reserve: look-back records");
  if (cudaMemset(p->d_records, 0, nrec * sizeof(unsigned long long)) != cudaSuccess)
    return cleanup(BG_ERR_CUDA, "bg_plan_reserve: clearing records");
  if (prog->desc.n_run > 0 &&
      cudaMalloc(&p->d_runs, (size_t)prog->desc.n_run * (size_t)max_tiles * sizeof(uint32_t)) != cudaSuccess)
    return cleanup(BG_ERR_NOMEM, "bg_plan_reserve: run masks");
  if (prog->desc.n_run > 0 &&
      cudaMalloc(&p->d_work, (size_t)work_words(prog->desc, max_tiles) * sizeof(uint32_t)) != cudaSuccess)
    return cleanup(BG_ERR_NOMEM, "bg_plan_reserve: work list");
  if (cudaMalloc(&p->d_state, 8 * sizeof(uint32_t)) != cudaSuccess)
    return cleanup(BG_ERR_NOMEM, "bg_plan_reserve: state");
  if (cudaMemset(p->d_state, 0, 8 * sizeof(uint32_t)) != cudaSuccess)
    return cleanup(BG_ERR_CUDA, "bg_plan_reserve: clearing state");
  *out = p;
  return BG_OK;
}

int bg_plan_set_layout(bg_plan *p, const bg_layout *L, void *stream) {
  if (!p || !layout_ok(L) || L->input_kind != p->layout.input_kind)
    return fail(BG_ERR_INVALID, "bg_plan_set_layout: bad layout");
  if (L->n_inputs > p->cap_inputs)
    return fail(BG_ERR_INVALID, "bg_plan_set_layout: more inputs than reserved");
  /* the staging buffer may still feed the previous upload */
  if (p->staged_pending) {
    if (cudaEventSynchronize(p->staged) != cudaSuccess)
      return fail(BG_ERR_CUDA, "bg_plan_set_layout: waiting for the previous upload");
    p->staged_pending = false;
  }
  const int64_t tiles = build_tables(p->prog, L, p->h_stage);
  if (tiles < 0) return (int)-tiles;
  if (tiles > p->cap_tiles)
    return fail(BG_ERR_INVALID, "bg_plan_set_layout: more tiles than reserved");
  const size_t ntab = 4 * (size_t)L->n_inputs + 1;
  cudaStream_t s = (cudaStream_t)stream;
  BG_CUDA(cudaMemcpyAsync(p->d_tables, p->h_stage, ntab * sizeof(int64_t), cudaMemcpyHostToDevice, s));
  BG_CUDA(cudaEventRecord(p->staged, s));
  p->staged_pending = true;
  p->layout = *L;
  p->layout.in_off = p->layout.in_len = p->layout.out_off = nullptr; /* not retained */
  p->n_tiles = tiles;
  const int warps_per_block = p->prog->desc.block / 32;
  const int64_t need = (tiles + warps_per_block - 1) / warps_per_block;
  p->grid = (int)std::max<int64_t>(
      1, std::min<int64_t>(need, (int64_t)sm_count() * p->prog->blocks_per_sm));
  return BG_OK;
}

int bg_plan_create(bg_program *prog, const bg_layout *L, bg_plan **out) {
  if (!prog || !out || !layout_ok(L)) return fail(BG_ERR_INVALID, "bg_plan_create: bad layout");
  *out = nullptr;
  std::vector<int64_t> tables(4 * (size_t)L->n_inputs + 1);
  const int64_t tiles = build_tables(prog, L, tables.data());
  if (tiles < 0) return (int)-tiles;
  if (tiles >= (int64_t)0xffffffffll) return fail(BG_ERR_INVALID, "bg_plan_create: too many tiles");
  bg_plan *p = nullptr;
  int rc = bg_plan_reserve(prog, L->input_kind, L->n_inputs, tiles, &p);
  if (rc != BG_OK) return rc;
  rc = bg_plan_set_layout(p, L, nullptr);
  if (rc == BG_OK && cudaStreamSynchronize(nullptr) != cudaSuccess) rc = fail(BG_ERR_CUDA, "bg_plan_create: upload");
  if (rc != BG_OK) {
    std::string keep = g_last_error;
    bg_plan_destroy(p);
    g_last_error = keep;
    return rc;
  }
  *out = p;
  return BG_OK;
}

int64_t bg_plan_tiles(const bg_plan *plan) { return plan ? plan->n_tiles : -1; }

int bg_plan_set_positions(bg_plan *plan, unsigned long long *positions, int64_t capacity) {
  if (!plan || capacity < 0 || capacity > ((int64_t)1 << 40))
    return fail(BG_ERR_INVALID, "bg_plan_set_positions: bad arguments");
  if (plan->prog->desc.n_outputs >= 4095 || plan->cap_inputs >= (1 << 20))
    return fail(BG_ERR_INVALID, "bg_plan_set_positions: more than 4094 outputs or 2^20 inputs");
  /* a program whose parts share outputs counts the bits it adds against the output streams;
   * for launches without them it keeps a set of the positions found so far, sized here at
   * twice the capacity (a power of two), allocated once and reused while it is big enough */
  if ((plan->prog->desc.flags & BG_PROGRAM_MERGES) && capacity > 0) {
    int64_t slots = 1024;
    while (slots < 2 * capacity) slots <<= 1;
    if (slots > plan->set_slots) {
      if (plan->d_set) cudaFree(plan->d_set);
      plan->d_set = nullptr;
      plan->set_slots = 0;
      if (cudaMalloc(&plan->d_set, (size_t)slots * sizeof(unsigned long long)) != cudaSuccess) {
        cudaGetLastError();
        return fail(BG_ERR_NOMEM, "bg_plan_set_positions: position set");
      }
      plan->set_slots = slots;
    }
  }
  plan->positions = capacity ? positions : nullptr;
  plan->pos_capacity = positions ? capacity : 0;
  plan->count_only = capacity > 0 && !positions;
  return BG_OK;
}

int bg_plan_positions_written(bg_plan *plan, void *stream, int64_t *written) {
  if (!plan || !written) return fail(BG_ERR_INVALID, "bg_plan_positions_written: bad arguments");
  unsigned long long v = 0;
  BG_CUDA(cudaMemcpyAsync(&v, plan->d_state + 6, sizeof v, cudaMemcpyDeviceToHost, (cudaStream_t)stream));
  BG_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
  *written = (int64_t)v;
  return BG_OK;
}

int bg_plan_stats(bg_plan *plan, void *stream, int32_t n_parts, int64_t *tiles_run, int64_t *rows) {
  if (!plan || n_parts < 0 || (n_parts > 0 && (!tiles_run || !rows)))
    return fail(BG_ERR_INVALID, "bg_plan_stats: bad arguments");
  const bg_program *prog = plan->prog;
  if (prog->desc.n_run <= 0 || !prog->pmask || !plan->d_runs || !plan->d_work)
    return fail(BG_ERR_INVALID, "bg_plan_stats: single-kernel program (every tile runs every term)");
  if (n_parts != prog->desc.n_parts) return fail(BG_ERR_INVALID, "bg_plan_stats: n_parts differs");
  const int64_t T = plan->n_tiles, NR = prog->desc.n_run, pmw = prog->pmw;
  std::vector<uint32_t> runs((size_t)(NR * T)), pm((size_t)(n_parts * pmw * 2)), cnt((size_t)n_parts);
  cudaStream_t s = (cudaStream_t)stream;
  if (!runs.empty())
    BG_CUDA(cudaMemcpyAsync(runs.data(), plan->d_runs, runs.size() * sizeof(uint32_t),
                            cudaMemcpyDeviceToHost, s));
  if (n_parts > 0) {
    BG_CUDA(cudaMemcpyAsync(pm.data(), prog->pmask, pm.size() * sizeof(uint32_t),
                            cudaMemcpyDeviceToHost, s));
    BG_CUDA(cudaMemcpyAsync(cnt.data(), plan->d_work + BG_WORK_HEAD, cnt.size() * sizeof(uint32_t),
                            cudaMemcpyDeviceToHost, s));
  }
  BG_CUDA(cudaStreamSynchronize(s));
  /* the execute pass runs part k on tile g when one of k's (word, mask) pairs meets the tile's
     run word, and walks the rows the work list holds for k */
  for (int32_t k = 0; k < n_parts; ++k) {
    int64_t n = 0;
    for (int64_t g = 0; g < T; ++g) {
      bool any = false;
      for (int64_t e = 0; e < pmw && !any; ++e) {
        const uint32_t w = pm[(size_t)((k * pmw + e) * 2)], m = pm[(size_t)((k * pmw + e) * 2 + 1)];
        any = m != 0u && w < (uint32_t)NR && (runs[(size_t)(w * T + g)] & m) != 0u;
      }
      n += any;
    }
    tiles_run[k] = n;
    rows[k] = (int64_t)cnt[(size_t)k];
  }
  return BG_OK;
}

int bg_plan_set_wait_limit(bg_plan *plan, int64_t spin_limit_cycles, int64_t debug_wait_tile) {
  if (!plan) return fail(BG_ERR_INVALID, "bg_plan_set_wait_limit: null plan");
  plan->spin_limit = spin_limit_cycles;
  plan->debug_wait_tile = debug_wait_tile;
  return BG_OK;
}

}  // extern "C"

/* Everything of one scan after its prologue: the carry pre-pass and its scan when the program
 * has one, then the main kernel.  All launches go to `s`, in this order. */
/* Tiles per warp chunk of the classify / pre-pass kernels for a launch of `tiles` tiles on
 * `warps` resident warps: whole rows of 32 tiles while they keep at least half of the warps
 * busy, else the longest shorter chunk (a power of two) that does, so that small launches
 * spread over the whole GPU instead of walking 32 tiles per warp. */
static int chunk_tiles_for(int64_t tiles, int64_t warps) {
  int ct = 32;
  while (ct > 1 && 2 * tiles < warps * ct) ct >>= 1;
  return ct;
}

/* Launch grid and chunk length of a classify / pre-pass kernel; with chunks shorter than a row
 * the row words they OR into (pre-pass bitmaps, and in the split form the row summaries) are
 * zeroed first. */
static int chunk_launch(const bg_program *prog, BgParams &prm, int block, int blocks_per_sm,
                        uint32_t *rowrun, cudaStream_t s, int &grid) {
  const int warps_per_block = block / 32;
  const int64_t resident = (int64_t)sm_count() * blocks_per_sm;
  prm.chunk_tiles = chunk_tiles_for(prm.n_tiles, resident * warps_per_block);
  const int64_t rows = (prm.n_tiles + 31) / 32;
  if (prm.chunk_tiles < 32) {
    if (prog->desc.n_pre > 0)
      BG_CUDA(cudaMemsetAsync(prm.pre_bits, 0,
                              sizeof(uint32_t) * 3 * (size_t)rows * (size_t)prog->desc.n_pre, s));
    if (rowrun)
      BG_CUDA(cudaMemsetAsync(rowrun, 0, sizeof(uint32_t) * (size_t)prog->desc.n_run * (size_t)rows,
                              s));
  }
  const int64_t chunks = (prm.n_tiles + prm.chunk_tiles - 1) / prm.chunk_tiles;
  const int64_t need = (chunks + warps_per_block - 1) / warps_per_block;
  grid = (int)std::max<int64_t>(1, std::min<int64_t>(need, resident));
  return BG_OK;
}

static int launch_passes(const bg_program *prog, BgParams &prm, int grid, cudaStream_t s) {
  void *args[] = {&prm};
  if (prog->cls_kernel) {
    /* split form: classify every tile (it also does the launch prologue, zeroes the output
     * words the parts OR into and writes every row's summary of run masks), scan the pre-pass
     * carries and list each part's rows with work (one launch), then run the parts */
    const int64_t rows = (prm.n_tiles + 31) / 32;
    if (!prog->pmask || prog->desc.n_parts > 4096)
      return fail(BG_ERR_INVALID, "split-form launch: no part table or more than 4096 parts");
    int cls_grid = 1;
    const int rc = chunk_launch(prog, prm, prog->cls_block, prog->pre_blocks_per_sm,
                                prm.work + BG_WORK_HEAD + (int64_t)prog->desc.n_parts * (1 + rows),
                                s, cls_grid);
    if (rc != BG_OK) return rc;
    BG_CUDA(cudaLaunchKernel((const void *)prog->cls_kernel, dim3(cls_grid),
                             dim3(prog->cls_block), args, (size_t)prog->cls_smem, s));
    /* the row kernel and execute are launched as programmatic dependents: each may be set up
     * while its predecessor drains, and waits (griddepcontrol.wait) before reading its results */
    cudaLaunchAttribute pdl;
    pdl.id = cudaLaunchAttributeProgrammaticStreamSerialization;
    pdl.val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.stream = s;
    cfg.attrs = &pdl;
    cfg.numAttrs = 1;
    const int n_parts = std::max(1, prog->desc.n_parts);
    /* 512 threads, two blocks per SM: one wave for up to 2 x SMs parts and additions */
    cfg.gridDim = dim3(prog->desc.n_pre + (rows <= WARP_LIST_ROWS ? (n_parts + 15) / 16 : n_parts));
    cfg.blockDim = dim3(512);
    BG_CUDA(cudaLaunchKernelEx(&cfg, bg_rows_kernel, prm.pre_bits, prm.n_tiles,
                               (const int64_t *)prm.tile_prefix, (int)prm.n_inputs,
                               (int)prog->desc.n_pre,
                               (const uint32_t *)(prm.work + BG_WORK_HEAD +
                                                  (int64_t)prog->desc.n_parts * (1 + rows)),
                               prog->pmask, prog->pmw, prm.work,
                               (int)std::max(1, prog->desc.n_parts), (int64_t)rows));
    /* persistent execute blocks: every resident slot for a large launch, no more warps than
     * tiles for a small one (its work items, (part, row) pairs, are fewer still) */
    const int64_t warps = prog->desc.block / 32;
    cfg.gridDim = dim3((unsigned)std::max<int64_t>(
        1, std::min<int64_t>((int64_t)sm_count() * prog->blocks_per_sm,
                             (prm.n_tiles + warps - 1) / warps)));
    cfg.blockDim = dim3(prog->desc.block);
    BG_CUDA(cudaLaunchKernelExC(&cfg, (const void *)prog->kernel, args));
    return BG_OK;
  }
  if (prog->pre_kernel) {
    int pre_grid = 1;
    const int rc = chunk_launch(prog, prm, prog->desc.block, prog->pre_blocks_per_sm, nullptr, s,
                                pre_grid);
    if (rc != BG_OK) return rc;
    BG_CUDA(cudaLaunchKernel((const void *)prog->pre_kernel, dim3(pre_grid),
                             dim3(prog->desc.block), args, 0, s));
    bg_carry_scan_kernel<<<prog->desc.n_pre, 1024, 0, s>>>(prm.pre_bits, prm.n_tiles,
                                                            prm.tile_prefix, prm.n_inputs);
    BG_CUDA(cudaGetLastError());
  }
  BG_CUDA(cudaLaunchKernel((const void *)prog->kernel, dim3(grid), dim3(prog->desc.block), args,
                           0, s));
  return BG_OK;
}

extern "C" {

int bg_plan_launch(bg_plan *plan, const void *input, uint32_t *out_streams,
                   unsigned long long *counts, void *stream) {
  if (!plan || !input) return fail(BG_ERR_INVALID, "bg_plan_launch: null plan or input");
  const bool use_set = !out_streams && (plan->prog->desc.flags & BG_PROGRAM_MERGES);
  if (use_set && (!plan->d_set || (!plan->positions && !plan->count_only)))
    return fail(BG_ERR_INVALID,
                "bg_plan_launch: this program merges outputs across parts: without out_streams "
                "it needs a position capacity (bg_plan_set_positions)");
  const bg_layout &L = plan->layout;
  if (L.input_kind == BG_INPUT_BYTES && !aligned16(input))
    return fail(BG_ERR_ALIGN, "bg_plan_launch: input not 16-byte aligned");
  cudaStream_t s = (cudaStream_t)stream;
  const int64_t n = L.n_inputs;
  BgParams prm{};
  prm.in_bytes = L.input_kind == BG_INPUT_BYTES ? (const uint8_t *)input : nullptr;
  prm.in_basis = L.input_kind == BG_INPUT_BASIS ? (const uint32_t *)input : nullptr;
  prm.in_off = plan->d_tables;
  prm.in_len = plan->d_tables + n;
  prm.tile_prefix = plan->d_tables + 2 * n;
  prm.out_off = plan->d_tables + 3 * n + 1;
  prm.out = out_streams;
  prm.counts = counts;
  prm.records = plan->d_records;
  prm.state = plan->d_state;
  prm.basis_stride = L.basis_stride;
  prm.out_stride = L.out_stride;
  prm.n_tiles = plan->n_tiles;
  prm.spin_limit = 2000000000ll; /* ~1 s at 2 GHz */
  prm.debug_wait_tile = plan->debug_wait_tile;
  prm.positions = plan->positions;
  prm.pos_capacity = plan->pos_capacity;
  prm.pos_set = use_set ? plan->d_set : nullptr;
  prm.pos_set_mask = use_set ? plan->set_slots - 1 : 0;
  prm.runs = plan->d_runs;
  /* the pre-pass bitmaps start after the records of the reserved tile count, so that a layout
   * with more tiles than the last one never finds bitmap words where it looks for records */
  prm.pre_bits = reinterpret_cast<uint32_t *>(plan->d_records +
                                              (int64_t)std::max(1, plan->prog->desc.n_adds) * plan->cap_tiles);
  prm.work = plan->d_work;
  if (plan->spin_limit > 0) prm.spin_limit = plan->spin_limit;
  prm.n_inputs = (int32_t)n;
  prm.input_kind = L.input_kind;
  if (!plan->prog->cls_kernel) { /* the split form's classify kernel does this itself */
    if (counts)
      BG_CUDA(cudaMemsetAsync(counts, 0,
                              sizeof(unsigned long long) * (size_t)plan->prog->desc.n_outputs * n, s));
    bg_prologue_kernel<<<1, 1, 0, s>>>(plan->d_state);
    BG_CUDA(cudaGetLastError());
  }
  return launch_passes(plan->prog, prm, plan->grid, s);
}

int bg_plan_sync(bg_plan *plan, void *stream) {
  if (!plan) return fail(BG_ERR_INVALID, "bg_plan_sync: null plan");
  BG_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
  uint32_t st = 0;
  BG_CUDA(cudaMemcpy(&st, plan->d_state + 1, sizeof st, cudaMemcpyDeviceToHost));
  if (st) {
    BG_CUDA(cudaMemset(plan->d_state + 1, 0, sizeof st));
    if (st & BG_DEV_ERR_TIMEOUT) return fail(BG_ERR_TIMEOUT, "carry look-back wait timed out");
    if (st & BG_DEV_ERR_SETFULL)
      return fail(BG_ERR_CAPACITY, "match positions exceeded twice the position capacity of a "
                                   "launch without output streams; counts are incomplete");
    if (st & BG_DEV_ERR_CAPACITY)
      return fail(BG_ERR_CAPACITY, "match positions exceeded the buffer; counts are complete");
    return fail(BG_ERR_DEVICE, "carry look-back walked past the start of its input");
  }
  return BG_OK;
}

int bg_plan_destroy(bg_plan *plan) {
  if (!plan) return BG_OK;
  if (plan->staged) {
    cudaEventSynchronize(plan->staged);
    cudaEventDestroy(plan->staged);
  }
  if (plan->d_tables) cudaFree(plan->d_tables);
  if (plan->d_records) cudaFree(plan->d_records);
  if (plan->d_state) cudaFree(plan->d_state);
  if (plan->d_runs) cudaFree(plan->d_runs);
  if (plan->d_work) cudaFree(plan->d_work);
  if (plan->d_set) cudaFree(plan->d_set);
  if (plan->h_stage) cudaFreeHost(plan->h_stage);
  delete plan;
  return BG_OK;
}

}  // extern "C"

/* ======================================================================================== */
/* Allocation-free scan of one byte input                                                  */
/* ======================================================================================== */
/* Some callers may not allocate device memory while they scan: a host whose device memory is
 * owned by a pooling allocator with a fixed budget, or a latency-bound loop where cudaFree's
 * device-wide synchronisation would stall other streams.  bg_scan_noalloc serves them with
 * the same fused kernel as bg_plan_launch.  The look-back records, the one-input launch tables
 * and the state words live in this fixed array, which the library's module carries.
 *
 * Layout in 64-bit words:
 *   [0, 4)    state: the eight 32-bit slots of a plan's state (tile counter, status, epoch,
 *             a record no kernel writes, match positions written);
 *   [4, 9)    tables of the one input: in_off, in_len, tile_prefix[0..1], out_off;
 *   [32, end) look-back records, [n_adds][n_tiles], the pre-pass bitmaps (3 words of 32
 *             tiles per pre-pass addition), then (split form) the run masks,
 *             [n_run][n_tiles] 32-bit words, and the work list.
 * The array starts zeroed when the module loads.  Every call clears the counters and the
 * status, bumps the epoch and zeroes its own record range [32, 32 + additions * tiles): that
 * range moves with the program and the input size, so it can cover words an earlier call used
 * as pre-pass bitmaps, run masks or work list, untagged values the look-back could take for a
 * record of this call's epoch.  Calls share the array, so calls that overlap on the GPU race
 * on it. */
namespace {

constexpr int64_t kNoallocWords = BG_NOALLOC_SCRATCH_BYTES / 8;
constexpr int64_t kNoallocRecordsAt = 32;
static_assert(kNoallocWords - kNoallocRecordsAt == (int64_t)BG_NOALLOC_RECORDS, "scratch layout");

static __device__ __align__(256) unsigned long long bg_noalloc_scratch[kNoallocWords];

constexpr int kNoallocMaxDevices = 64;
std::mutex g_noalloc_mu;
unsigned long long *g_noalloc_ptr[kNoallocMaxDevices] = {};

/* Clears what must start at zero for one call and writes the one-input tables. */
__global__ void bg_noalloc_prologue_kernel(unsigned long long *scratch, int64_t n_bytes,
                                           int64_t n_tiles, unsigned long long *counts,
                                           int n_counts) {
  if (threadIdx.x == 0) {
    uint32_t *state = reinterpret_cast<uint32_t *>(scratch);
    state[0] = 0u; /* tile counter */
    state[1] = 0u; /* status */
    scratch[1] += 1ull; /* epoch (state[2..3]) */
    scratch[2] = 0ull;  /* the never-written record (state[4..5]) */
    scratch[3] = 0ull;  /* match positions written (state[6..7]) */
    int64_t *t = reinterpret_cast<int64_t *>(scratch + 4);
    t[0] = 0;       /* in_off */
    t[1] = n_bytes; /* in_len */
    t[2] = 0;       /* tile_prefix[0] */
    t[3] = n_tiles; /* tile_prefix[1] */
    t[4] = 0;       /* out_off */
  }
  if (counts)
    for (int i = threadIdx.x; i < n_counts; i += blockDim.x) counts[i] = 0ull;
}

/* Hands the scan's status bits to the caller's word. */
__global__ void bg_noalloc_epilogue_kernel(const unsigned long long *scratch, uint32_t *status) {
  *status = reinterpret_cast<const uint32_t *>(scratch)[1];
}

/* Device address of the array on the current device, looked up once per device. */
int noalloc_scratch(unsigned long long **out) {
  int dev = -1;
  BG_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kNoallocMaxDevices)
    return fail(BG_ERR_INVALID, "bg_scan_noalloc: device ordinal beyond 63");
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    unsigned long long *ptr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress((void **)&ptr, bg_noalloc_scratch);
    if (e != cudaSuccess || !ptr)
      return fail(BG_ERR_CUDA, std::string("bg_scan_noalloc: cudaGetSymbolAddress of the scratch: ") +
                                   cudaGetErrorString(e));
    g_noalloc_ptr[dev] = ptr;
  }
  *out = g_noalloc_ptr[dev];
  return BG_OK;
}

}  // namespace

extern "C" int bg_scan_noalloc(const bg_program *prog, const uint8_t *input, int64_t n_bytes,
                               uint32_t *out_streams, int64_t out_stride,
                               unsigned long long *counts, uint32_t *status, void *stream) {
  if (!prog || !prog->kernel || !input || !status || n_bytes < 0)
    return fail(BG_ERR_INVALID, "bg_scan_noalloc: null program, input or status, or negative size");
  if (!aligned16(input)) return fail(BG_ERR_ALIGN, "bg_scan_noalloc: input not 16-byte aligned");
  if (!out_streams && (prog->desc.flags & BG_PROGRAM_MERGES))
    return fail(BG_ERR_INVALID,
                "bg_scan_noalloc: this program merges outputs across parts and needs out_streams");
  const int64_t W = (n_bytes + 31) / 32;
  if (out_streams && out_stride < W)
    return fail(BG_ERR_INVALID, "bg_scan_noalloc: out_stride shorter than the input's words");
  const int64_t tile_words =
      (int64_t)(32 - prog->desc.halo_lanes - prog->desc.tail_lanes) * prog->desc.wpt;
  const int64_t tiles = std::max<int64_t>(1, (W + tile_words - 1) / tile_words);
  const int64_t adds = std::max(1, prog->desc.n_adds);
  /* 64-bit scratch words: the look-back records and pre-pass bitmaps, then the run masks */
  auto scratch_words = [&](int64_t n) {
    return record_words(prog->desc, n) + ((int64_t)prog->desc.n_run * n + 1) / 2 +
           (work_words(prog->desc, n) + 1) / 2;
  };
  if (scratch_words(tiles) > (int64_t)BG_NOALLOC_RECORDS) {
    int64_t lo = 0, hi = tiles; /* largest tile count that fits */
    while (hi - lo > 1) {
      const int64_t m = (lo + hi) / 2;
      if (scratch_words(m) <= (int64_t)BG_NOALLOC_RECORDS) lo = m; else hi = m;
    }
    char msg[360];
    snprintf(msg, sizeof msg,
             "bg_scan_noalloc: %lld bytes span %lld tiles of %lld words and need %lld scratch "
             "words (%lld additions, %d pre-pass, %d run-mask words per tile); the fixed %u-byte "
             "scratch holds %u, so at most %lld tiles (%lld bytes) for this program",
             (long long)n_bytes, (long long)tiles, (long long)tile_words,
             (long long)scratch_words(tiles), (long long)adds, prog->desc.n_pre, prog->desc.n_run,
             (unsigned)BG_NOALLOC_SCRATCH_BYTES, (unsigned)BG_NOALLOC_RECORDS, (long long)lo,
             (long long)lo * tile_words * 32);
    return fail(BG_ERR_CAPACITY, msg);
  }
  unsigned long long *scratch = nullptr;
  const int rc = noalloc_scratch(&scratch);
  if (rc != BG_OK) return rc;

  cudaStream_t s = (cudaStream_t)stream;
  BgParams prm{};
  prm.in_bytes = input;
  prm.in_basis = nullptr;
  const int64_t *tables = reinterpret_cast<const int64_t *>(scratch + 4);
  prm.in_off = tables;
  prm.in_len = tables + 1;
  prm.tile_prefix = tables + 2;
  prm.out_off = tables + 4;
  prm.out = out_streams;
  prm.counts = counts;
  prm.records = scratch + kNoallocRecordsAt;
  prm.state = reinterpret_cast<uint32_t *>(scratch);
  prm.pre_bits = reinterpret_cast<uint32_t *>(scratch + kNoallocRecordsAt + adds * tiles);
  prm.runs = prog->desc.n_run > 0
                 ? reinterpret_cast<uint32_t *>(scratch + kNoallocRecordsAt +
                                                record_words(prog->desc, tiles))
                 : nullptr;
  prm.work = prog->desc.n_run > 0
                 ? reinterpret_cast<uint32_t *>(scratch + kNoallocRecordsAt +
                                                record_words(prog->desc, tiles) +
                                                ((int64_t)prog->desc.n_run * tiles + 1) / 2)
                 : nullptr;
  prm.positions = nullptr;
  prm.pos_capacity = 0;
  prm.pos_set = nullptr;
  prm.pos_set_mask = 0;
  prm.basis_stride = 0;
  prm.out_stride = out_stride;
  prm.n_tiles = tiles;
  prm.spin_limit = 2000000000ll; /* ~1 s at 2 GHz */
  prm.debug_wait_tile = -1;
  prm.n_inputs = 1;
  prm.input_kind = BG_INPUT_BYTES;
  const int warps_per_block = prog->desc.block / 32;
  const int64_t need = (tiles + warps_per_block - 1) / warps_per_block;
  const int grid = (int)std::max<int64_t>(
      1, std::min<int64_t>(need, (int64_t)sm_count() * prog->blocks_per_sm));

  bg_noalloc_prologue_kernel<<<1, 256, 0, s>>>(scratch, n_bytes, tiles, counts,
                                               prog->desc.n_outputs);
  BG_CUDA(cudaGetLastError());
  /* a zero word is an unpublished record of every epoch (a memset allocates nothing) */
  BG_CUDA(cudaMemsetAsync(prm.records, 0, sizeof(unsigned long long) * (size_t)(adds * tiles), s));
  const int lrc = launch_passes(prog, prm, grid, s);
  if (lrc != BG_OK) return lrc;
  bg_noalloc_epilogue_kernel<<<1, 1, 0, s>>>(scratch, status);
  BG_CUDA(cudaGetLastError());
  return BG_OK;
}
