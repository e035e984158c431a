/* Whole-stream executor for Pablo programs that keep while / if blocks.
 *
 * The reference evaluates a Pablo `while v:` per CTA tile inside its fused kernel
 * (bitgen/inst/inst_block_while.py:50-133, block_all_zeros at template.cu:356-374), which gives
 * tile-local rather than whole-stream conditions.  Its Python and torch lowerings state the
 * intended semantics: the body runs again while any bit of v is set anywhere in the stream
 * (inst_block_while.py:137-153; inst_block_if.py:314-342).  This executor implements exactly
 * that: every instruction is one kernel over the whole stream of one input, and a loop / branch
 * condition is reduced over the whole stream and read back by the host.
 *
 * Additions run as a three-kernel carry scan: per-block (generate, propagate) aggregates, a
 * warp-parallel scan of the block aggregates, and an apply pass that adds with the exact carry.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <vector>

#include "../../include/bitgen_gb300.h"
#include "bg_transpose.cuh"

extern "C" int bg_interp_fail(int code, const char *msg);

namespace {

constexpr int T = 256; /* threads (= words) per block */
constexpr unsigned FULL = 0xffffffffu;

enum { OP_AND = 0, OP_OR, OP_XOR, OP_NOT, OP_SEL, OP_ADV, OP_MATCHSTAR, OP_SCANTHRU, OP_COPY,
       OP_WHILE, OP_IF, OP_LOOK };

__global__ void k_bitwise(int op, uint32_t *__restrict__ d, const uint32_t *__restrict__ a,
                          const uint32_t *__restrict__ b, const uint32_t *__restrict__ c,
                          int64_t W) {
  for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < W;
       w += (int64_t)gridDim.x * blockDim.x) {
    uint32_t r;
    switch (op) {
      case OP_AND: r = a[w] & b[w]; break;
      case OP_OR: r = a[w] | b[w]; break;
      case OP_XOR: r = a[w] ^ b[w]; break;
      case OP_NOT: r = ~a[w]; break;
      case OP_SEL: r = (a[w] & b[w]) | (~a[w] & c[w]); break;
      default: r = a[w]; break;
    }
    d[w] = r;
  }
}

__global__ void k_fill(uint32_t *d, uint32_t v, int64_t W) {
  for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < W;
       w += (int64_t)gridDim.x * blockDim.x)
    d[w] = v;
}

/* Advance(a, shift): character p moves to p + shift; MSB-first words. */
__global__ void k_advance(uint32_t *__restrict__ d, const uint32_t *__restrict__ a, int64_t shift,
                          int64_t W) {
  const int64_t q = shift / 32;
  const int r = (int)(shift % 32);
  for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < W;
       w += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t cur = (w - q >= 0) ? a[w - q] : 0u;
    const uint32_t prev = (w - q - 1 >= 0) ? a[w - q - 1] : 0u;
    d[w] = r == 0 ? cur : __funnelshift_r(cur, prev, r);
  }
}

/* Lookahead(a, shift): character p takes a[p + shift]; positions >= n read as 0. */
__global__ void k_lookahead(uint32_t *__restrict__ d, const uint32_t *__restrict__ a, int64_t shift,
                            int64_t W, int64_t n) {
  const int64_t q = shift / 32;
  const int r = (int)(shift % 32);
  for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < W;
       w += (int64_t)gridDim.x * blockDim.x) {
    uint32_t v[2];
    for (int k = 0; k < 2; ++k) {
      const int64_t i = w + q + k;
      uint32_t x = i < W ? a[i] : 0u;
      const int64_t rem = n - 32 * i;
      if (rem <= 0) x = 0u;
      else if (rem < 32) x &= FULL << (32 - rem);
      v[k] = x;
    }
    d[w] = r == 0 ? v[0] : __funnelshift_l(v[1], v[0], r);
  }
}

/* any bit set at a position < n */
__global__ void k_any(const uint32_t *__restrict__ a, int64_t W, int64_t n, uint32_t *flag) {
  uint32_t o = 0;
  for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < W;
       w += (int64_t)gridDim.x * blockDim.x) {
    uint32_t v = a[w];
    const int64_t rem = n - 32 * w;
    if (rem < 32) v &= FULL << (32 - rem);
    o |= v;
  }
  if (__any_sync(FULL, o != 0u) && (threadIdx.x & 31) == 0) atomicOr(flag, 1u);
}

/* operands of the addition in increasing significance order */
__device__ __forceinline__ void add_operands(int op, uint32_t m, uint32_t c, uint32_t &x,
                                             uint32_t &y) {
  x = __brev(op == OP_MATCHSTAR ? (m & c) : m);
  y = __brev(c);
}

/* block-level carries: returns the carry into this thread's word; block cin given. */
__device__ uint32_t block_carry(uint32_t g, uint32_t p, uint32_t cin, uint32_t *outG,
                                uint32_t *outP) {
  __shared__ uint32_t sG[T / 32], sP[T / 32], sC[T / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t Gm = __ballot_sync(FULL, g), Pm = __ballot_sync(FULL, p);
  const uint32_t A = Gm | Pm, B = Gm;
  if (lane == 0) {
    sG[warp] = (uint32_t)(((unsigned long long)A + B) >> 32);
    sP[warp] = Pm == FULL ? 1u : 0u;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t c = cin, G = 0, P = 1;
    for (int i = 0; i < T / 32; ++i) {
      sC[i] = c;
      c = sG[i] | (sP[i] & c);
      G = sG[i] | (sP[i] & G);
      P &= sP[i];
    }
    if (outG) *outG = G;
    if (outP) *outP = P;
  }
  __syncthreads();
  const uint32_t cw = sC[warp];
  const uint32_t cvec = (uint32_t)((unsigned long long)A + B + cw) ^ A ^ B;
  return (cvec >> lane) & 1u;
}

__global__ void __launch_bounds__(T) k_add_agg(int op, const uint32_t *__restrict__ m,
                                               const uint32_t *__restrict__ c, int64_t W,
                                               uint2 *agg) {
  const int64_t w = (int64_t)blockIdx.x * T + threadIdx.x;
  uint32_t x = 0, y = 0;
  if (w < W) add_operands(op, m[w], c[w], x, y);
  const uint32_t s = x + y;
  uint32_t G = 0, P = 0;
  (void)block_carry(s < x ? 1u : 0u, s == FULL ? 1u : 0u, 0u, &G, &P);
  if (threadIdx.x == 0) agg[blockIdx.x] = make_uint2(G, P);
}

/* exclusive carry scan over block aggregates, one warp, 32 blocks per step */
__global__ void k_add_scan(uint2 *agg, int64_t nb) {
  const int lane = threadIdx.x;
  uint32_t cin = 0;
  for (int64_t base = 0; base < nb; base += 32) {
    const int64_t i = base + lane;
    const uint2 a = i < nb ? agg[i] : make_uint2(0u, 0u);
    const uint32_t Gm = __ballot_sync(FULL, a.x), Pm = __ballot_sync(FULL, a.y);
    const uint32_t A = Gm | Pm, B = Gm;
    const unsigned long long sum = (unsigned long long)A + B + cin;
    const uint32_t cvec = (uint32_t)sum ^ A ^ B;
    if (i < nb) agg[i].x = (cvec >> lane) & 1u;
    /* carry out of the last valid block of this step */
    const int last = (nb - 1 - base) < 31 ? (int)(nb - 1 - base) : 31;
    const uint32_t lastc = __shfl_sync(FULL, (cvec >> lane) & 1u, last);
    const uint2 la = make_uint2(__shfl_sync(FULL, a.x, last), __shfl_sync(FULL, a.y, last));
    cin = la.x | (la.y & lastc);
  }
}

__global__ void __launch_bounds__(T) k_add_apply(int op, uint32_t *__restrict__ d,
                                                 const uint32_t *__restrict__ m,
                                                 const uint32_t *__restrict__ c, int64_t W,
                                                 const uint2 *__restrict__ agg) {
  const int64_t w = (int64_t)blockIdx.x * T + threadIdx.x;
  uint32_t x = 0, y = 0, mm = 0, cc = 0;
  if (w < W) {
    mm = m[w];
    cc = c[w];
    add_operands(op, mm, cc, x, y);
  }
  const uint32_t s = x + y;
  const uint32_t carry =
      block_carry(s < x ? 1u : 0u, s == FULL ? 1u : 0u, agg[blockIdx.x].x, nullptr, nullptr);
  if (w < W) {
    const uint32_t sum = __brev(s + carry);
    d[w] = op == OP_MATCHSTAR ? ((sum ^ cc) | mm) : (sum & ~cc);
  }
}

/* transpose of one input with a ragged tail (bytes beyond n read as 0) */
__global__ void k_transpose_input(const uint8_t *__restrict__ src, int64_t n, uint32_t *basis,
                                  int64_t W, int64_t stride) {
  for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < W;
       w += (int64_t)gridDim.x * blockDim.x) {
    uint32_t u[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    const int64_t rem = n - 32 * w;
    if (rem >= 32) {
      const uint4 *q = reinterpret_cast<const uint4 *>(src + 32 * w);
      const uint4 a = q[0], b = q[1];
      u[0] = a.x; u[1] = a.y; u[2] = a.z; u[3] = a.w;
      u[4] = b.x; u[5] = b.y; u[6] = b.z; u[7] = b.w;
    } else {
      for (int64_t k = 0; k < rem; ++k) u[k >> 2] |= (uint32_t)src[32 * w + k] << (8 * (k & 3));
    }
    uint32_t o[8];
    bg::transpose32(u, o);
    for (int i = 0; i < 8; ++i) basis[i * stride + w] = o[i];
  }
}

__global__ void k_store(const uint32_t *__restrict__ v, uint32_t *out, int64_t W, int64_t n,
                        unsigned long long *count) {
  uint32_t cnt = 0;
  for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < W;
       w += (int64_t)gridDim.x * blockDim.x) {
    uint32_t x = v[w];
    const int64_t rem = n - 32 * w;
    if (rem < 32) x &= FULL << (32 - rem);
    if (out) out[w] = x;
    cnt += __popc(x);
  }
  for (int d = 16; d > 0; d >>= 1) cnt += __shfl_xor_sync(FULL, cnt, d);
  if (count && (threadIdx.x & 31) == 0 && cnt) atomicAdd(count, (unsigned long long)cnt);
}

int grid_for(int64_t W) { return (int)std::max<int64_t>(1, std::min<int64_t>((W + T - 1) / T, 4096)); }

}  // namespace

struct bg_interp {
  std::vector<bg_instr> code;
  int n_slots = 0;
  std::vector<int> outs;
};

namespace {

struct Exec {
  bg_interp *P;
  std::vector<uint32_t *> slot;
  int64_t W, n;
  uint2 *agg;
  uint32_t *flag;
  cudaStream_t s;
  int64_t max_iter;
  int status = BG_OK;
  std::string err;

  bool any(int sl) {
    if (cudaMemsetAsync(flag, 0, 4, s) != cudaSuccess) return fail_cuda();
    k_any<<<grid_for(W), T, 0, s>>>(slot[sl], W, n, flag);
    uint32_t h = 0;
    if (cudaMemcpyAsync(&h, flag, 4, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      return fail_cuda();
    return h != 0;
  }
  bool fail_cuda() {
    if (status == BG_OK) {
      status = BG_ERR_CUDA;
      err = cudaGetErrorString(cudaGetLastError());
    }
    return false;
  }

  void run(int64_t pc, int64_t end) {
    while (pc < end && status == BG_OK) {
      const bg_instr &I = P->code[pc];
      switch (I.op) {
        case OP_AND: case OP_OR: case OP_XOR: case OP_NOT: case OP_SEL: case OP_COPY:
          k_bitwise<<<grid_for(W), T, 0, s>>>(I.op, slot[I.dst], slot[I.a],
                                              I.b >= 0 ? slot[I.b] : nullptr,
                                              I.c >= 0 ? slot[I.c] : nullptr, W);
          ++pc;
          break;
        case OP_ADV:
          if (I.dst == I.a) { /* in-place shift needs a copy first */
            status = BG_ERR_INVALID;
            err = "Advance must not write its own operand";
            return;
          }
          k_advance<<<grid_for(W), T, 0, s>>>(slot[I.dst], slot[I.a], I.shift, W);
          ++pc;
          break;
        case OP_LOOK:
          if (I.dst == I.a) {
            status = BG_ERR_INVALID;
            err = "Lookahead must not write its own operand";
            return;
          }
          k_lookahead<<<grid_for(W), T, 0, s>>>(slot[I.dst], slot[I.a], I.shift, W, n);
          ++pc;
          break;
        case OP_MATCHSTAR: case OP_SCANTHRU: {
          const int64_t nb = (W + T - 1) / T;
          k_add_agg<<<(unsigned)nb, T, 0, s>>>(I.op, slot[I.a], slot[I.b], W, agg);
          k_add_scan<<<1, 32, 0, s>>>(agg, nb);
          k_add_apply<<<(unsigned)nb, T, 0, s>>>(I.op, slot[I.dst], slot[I.a], slot[I.b], W, agg);
          ++pc;
          break;
        }
        case OP_WHILE: {
          const int64_t body = pc + 1, bend = pc + 1 + I.shift;
          int64_t it = 0;
          while (status == BG_OK && any(I.a)) {
            if (max_iter > 0 && ++it > max_iter) {
              status = BG_ERR_TIMEOUT;
              err = "while loop exceeded the iteration bound";
              return;
            }
            run(body, bend);
          }
          pc = bend;
          break;
        }
        case OP_IF: {
          const int64_t t0 = pc + 1, t1 = t0 + I.shift, e1 = t1 + I.b;
          if (any(I.a)) run(t0, t1); else run(t1, e1);
          pc = e1;
          break;
        }
        default:
          status = BG_ERR_INVALID;
          err = "unknown instruction";
          return;
      }
      if (status == BG_OK && cudaPeekAtLastError() != cudaSuccess) fail_cuda();
    }
  }
};

}  // namespace

extern "C" {

int bg_interp_create(const bg_instr *code, int32_t n_code, int32_t n_slots,
                     const int32_t *out_slots, int32_t n_outputs, bg_interp **out) {
  if (!code || n_code < 0 || n_slots < 10 || !out || (n_outputs > 0 && !out_slots))
    return bg_interp_fail(BG_ERR_INVALID, "bg_interp_create: bad arguments");
  for (int32_t i = 0; i < n_code; ++i) {
    const bg_instr &I = code[i];
    auto bad = [&](int v) { return v < -1 || v >= n_slots; };
    if (I.op < 0 || I.op > OP_LOOK || bad(I.dst) || bad(I.a) || bad(I.b) || bad(I.c) ||
        ((I.op <= OP_COPY || I.op == OP_LOOK) && (I.dst < 10 || I.a < 0)) || I.shift < 0 ||
        ((I.op == OP_AND || I.op == OP_OR || I.op == OP_XOR || I.op == OP_MATCHSTAR ||
          I.op == OP_SCANTHRU) && I.b < 0) || (I.op == OP_SEL && (I.b < 0 || I.c < 0)) ||
        (I.op == OP_WHILE && i + 1 + (int64_t)I.shift > n_code) ||
        (I.op == OP_IF && i + 1 + (int64_t)I.shift + I.b > n_code))
      return bg_interp_fail(BG_ERR_INVALID, "bg_interp_create: bad instruction");
  }
  for (int32_t o = 0; o < n_outputs; ++o)
    if (out_slots[o] < 0 || out_slots[o] >= n_slots)
      return bg_interp_fail(BG_ERR_INVALID, "bg_interp_create: bad output slot");
  bg_interp *p = new bg_interp();
  p->code.assign(code, code + n_code);
  p->n_slots = n_slots;
  p->outs.assign(out_slots, out_slots + n_outputs);
  *out = p;
  return BG_OK;
}

int bg_interp_run(bg_interp *prog, const bg_layout *L, const void *input, uint32_t *out_streams,
                  unsigned long long *counts, int64_t max_iterations, void *stream) {
  if (!prog || !L || !input || L->n_inputs < 1 || !L->in_off || !L->in_len || !L->out_off)
    return bg_interp_fail(BG_ERR_INVALID, "bg_interp_run: bad arguments");
  cudaStream_t s = (cudaStream_t)stream;
  const int n_out = (int)prog->outs.size();
  int64_t Wmax = 1;
  for (int i = 0; i < L->n_inputs; ++i) {
    if (L->in_len[i] < 0) return bg_interp_fail(BG_ERR_INVALID, "bg_interp_run: negative length");
    if (L->input_kind == BG_INPUT_BYTES && ((uintptr_t)input + L->in_off[i]) % 16)
      return bg_interp_fail(BG_ERR_ALIGN, "bg_interp_run: input not 16-byte aligned");
    Wmax = std::max<int64_t>(Wmax, (L->in_len[i] + 31) / 32);
  }
  const int64_t nb = (Wmax + T - 1) / T;
  uint32_t *pool = nullptr;
  uint2 *agg = nullptr;
  uint32_t *flag = nullptr;
  const size_t pool_words = (size_t)prog->n_slots * (size_t)Wmax;
  if (cudaMalloc(&pool, pool_words * 4) != cudaSuccess ||
      cudaMalloc(&agg, (size_t)nb * sizeof(uint2)) != cudaSuccess ||
      cudaMalloc(&flag, 4) != cudaSuccess) {
    cudaFree(pool);
    cudaFree(agg);
    cudaFree(flag);
    cudaGetLastError();
    return bg_interp_fail(BG_ERR_NOMEM, "bg_interp_run: device memory");
  }
  if (counts && cudaMemsetAsync(counts, 0, sizeof(unsigned long long) * n_out * L->n_inputs, s) !=
                    cudaSuccess)
    return bg_interp_fail(BG_ERR_CUDA, "bg_interp_run: clearing counts");
  int rc = BG_OK;
  std::string msg;
  for (int i = 0; i < L->n_inputs && rc == BG_OK; ++i) {
    Exec e;
    e.P = prog;
    e.n = L->in_len[i];
    e.W = std::max<int64_t>(1, (e.n + 31) / 32);
    e.agg = agg;
    e.flag = flag;
    e.s = s;
    e.max_iter = max_iterations;
    e.slot.resize(prog->n_slots);
    for (int k = 0; k < prog->n_slots; ++k) e.slot[k] = pool + (size_t)k * Wmax;
    if (L->input_kind == BG_INPUT_BASIS) {
      const uint32_t *b = (const uint32_t *)input + L->in_off[i];
      for (int k = 0; k < 8; ++k)
        cudaMemcpyAsync(e.slot[k], b + k * L->basis_stride, e.W * 4, cudaMemcpyDeviceToDevice, s);
    } else {
      k_transpose_input<<<grid_for(e.W), T, 0, s>>>((const uint8_t *)input + L->in_off[i], e.n,
                                                    e.slot[0], e.W, Wmax);
    }
    k_fill<<<grid_for(e.W), T, 0, s>>>(e.slot[8], 0u, e.W);
    k_fill<<<grid_for(e.W), T, 0, s>>>(e.slot[9], FULL, e.W);
    e.run(0, (int64_t)prog->code.size());
    if (e.status != BG_OK) {
      rc = e.status;
      msg = e.err;
      break;
    }
    for (int o = 0; o < n_out; ++o) {
      uint32_t *dst = out_streams ? out_streams + o * L->out_stride + L->out_off[i] : nullptr;
      k_store<<<grid_for(e.W), T, 0, s>>>(e.slot[prog->outs[o]], dst, e.W, e.n,
                                          counts ? counts + (int64_t)o * L->n_inputs + i : nullptr);
    }
    if (cudaPeekAtLastError() != cudaSuccess) {
      rc = BG_ERR_CUDA;
      msg = cudaGetErrorString(cudaGetLastError());
    }
  }
  if (cudaStreamSynchronize(s) != cudaSuccess && rc == BG_OK) {
    rc = BG_ERR_CUDA;
    msg = cudaGetErrorString(cudaGetLastError());
  }
  cudaFree(pool);
  cudaFree(agg);
  cudaFree(flag);
  if (rc != BG_OK) return bg_interp_fail(rc, msg.c_str());
  return BG_OK;
}

int bg_interp_destroy(bg_interp *prog) {
  delete prog;
  return BG_OK;
}

}  // extern "C"
