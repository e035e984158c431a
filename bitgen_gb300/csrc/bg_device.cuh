/* Device library for generated bitstream programs (compiled by NVRTC for sm_103a).
 *
 * Stream layout (the reference's, bitgen/bitstream.py:228-258 and
 * bitgen/template/cuda/kernel.cu:60-100): a stream is a sequence of 32-bit words, character
 * 32*w + j at bit 31 - j of word w.  Advance moves marks to higher character positions, i.e.
 * toward the low bits of a word and then into the next word.
 *
 * Execution model: a warp owns a tile.  Lane l holds words [l*WPT, l*WPT + WPT) of the tile in
 * registers (type S).  Lanes [0, HL) are a halo: they re-compute the last HL*WPT words of the
 * previous tile so that every Advance of the program finds its source words inside the warp.
 * Lanes [32-TL, 32) are a tail halo for Lookahead, which reads later positions.  Lanes
 * [HL, 32-TL) are written out.  The generated kernel defines BG_WPT, BG_HL and BG_TL before
 * including this file.
 *
 * Additions (MatchStar, ScanThru) need the exact carry entering the tile.  For addition k the
 * carry is injected at lane DL_k, the first lane where both addends are exact.  If the addition
 * does not propagate through that lane the carry cannot change anything downstream and it is
 * resolved locally; otherwise the predecessor tile (which computed the same lane and knows it
 * is needed) publishes its carry-out, first as a (generate, propagate) aggregate and then as
 * an inclusive carry, and this tile reads it with a decoupled look-back.  Every wait is bounded
 * by a clock64 budget; on timeout the kernel records BG_DEV_ERR_TIMEOUT and continues.
 *
 * Additions over a wide class (such as '.', which covers whole tiles of text without line
 * breaks) would make every tile walk the look-back: their carries chain through the entire
 * input.  The first BG_NPRE additions of a program are of that kind and depend on no other
 * addition; for them a separate pass (the generated pre-pass or classify kernel, then the
 * runtime's carry scan) computes every tile's carry-in before the main kernel runs, which then
 * reads it (add_known) instead of waiting.
 */
#pragma once
#include "bg_params.h"
#include "bg_transpose.cuh"

#ifndef BG_WPT
#error "BG_WPT must be defined"
#endif
#ifndef BG_HL
#error "BG_HL must be defined"
#endif
#ifndef BG_TL
#define BG_TL 0
#endif
#ifndef BG_LOOKBACK_INLINE
#define BG_LOOKBACK_INLINE 0
#endif
#ifndef BG_LBK
#define BG_LBK 1 /* look-back records per lane per step */
#endif
#ifndef BG_LB_SPIN
#define BG_LB_SPIN 0 /* look-back polls before the first sleep */
#endif
#ifndef BG_NPRE
#define BG_NPRE 0 /* additions whose carries are computed by the pre-pass (numbered first) */
#endif
#ifndef BG_NRUN
#define BG_NRUN 1 /* words of the per-tile run mask (q-gram prefilter) */
#endif
#ifndef BG_BLOOM_BITS
#define BG_BLOOM_BITS 16 /* log2 of the prefilter's Bloom bitmap size */
#endif

namespace bg {

constexpr unsigned FULL = 0xffffffffu;
constexpr int WPT = BG_WPT;
constexpr int HL = BG_HL;
constexpr int TL = BG_TL;                   /* tail halo lanes (for Lookahead)     */
constexpr int SL = 32 - HL - TL;            /* output lanes per tile               */
constexpr long long SW = (long long)SL * WPT; /* output words per tile             */
constexpr int NPRE = BG_NPRE;
constexpr int NPRE_WORDS = NPRE > 0 ? (NPRE + 31) / 32 : 1;
static_assert(HL >= 0 && TL >= 0 && HL + TL < 32, "halos must leave output lanes");

struct S {
  uint32_t w[WPT];
};

// Low word of (hi:lo) >> R, as __funnelshift_r(lo, hi, R).  Written as a volatile instruction
// so that a shifted character class is recomputed where it is used (one instruction) rather
// than merged with its other uses and held in a register across the whole part.
template <int R>
__device__ __forceinline__ uint32_t shr_funnel(uint32_t lo, uint32_t hi) {
  uint32_t d;
  asm volatile("shf.r.wrap.b32 %0, %1, %2, %3;" : "=r"(d) : "r"(lo), "r"(hi), "n"(R));
  return d;
}

__device__ __forceinline__ S zero() {
  S r;
#pragma unroll
  for (int j = 0; j < WPT; ++j) r.w[j] = 0u;
  return r;
}
__device__ __forceinline__ S ones() {
  S r;
#pragma unroll
  for (int j = 0; j < WPT; ++j) r.w[j] = FULL;
  return r;
}
__device__ __forceinline__ S operator&(const S &a, const S &b) {
  S r;
#pragma unroll
  for (int j = 0; j < WPT; ++j) r.w[j] = a.w[j] & b.w[j];
  return r;
}
__device__ __forceinline__ S operator|(const S &a, const S &b) {
  S r;
#pragma unroll
  for (int j = 0; j < WPT; ++j) r.w[j] = a.w[j] | b.w[j];
  return r;
}
__device__ __forceinline__ S operator^(const S &a, const S &b) {
  S r;
#pragma unroll
  for (int j = 0; j < WPT; ++j) r.w[j] = a.w[j] ^ b.w[j];
  return r;
}
__device__ __forceinline__ S operator~(const S &a) {
  S r;
#pragma unroll
  for (int j = 0; j < WPT; ++j) r.w[j] = ~a.w[j];
  return r;
}
__device__ __forceinline__ S &operator|=(S &a, const S &b) {
#pragma unroll
  for (int j = 0; j < WPT; ++j) a.w[j] |= b.w[j];
  return a;
}
/* SEL(c, a, b) = (c & a) | (~c & b)   (bitgen/inst/inst_sel.py:42-57) */
__device__ __forceinline__ S sel(const S &c, const S &a, const S &b) {
  S r;
#pragma unroll
  for (int j = 0; j < WPT; ++j) r.w[j] = (c.w[j] & a.w[j]) | (~c.w[j] & b.w[j]);
  return r;
}
/* warp-wide "any bit set" (zero-block skipping test) */
__device__ __forceinline__ bool any(const S &x) {
  uint32_t o = 0;
#pragma unroll
  for (int j = 0; j < WPT; ++j) o |= x.w[j];
  return __any_sync(FULL, o != 0u);
}

/* word (lane*WPT + J) of the tile as seen from this lane, J may be negative (earlier lanes). */
__device__ __forceinline__ uint32_t word_back(const S &x, int J) {
  if (J >= 0) return x.w[J];
  const int L = (-J + WPT - 1) / WPT;
  const int I = J + L * WPT;
  return __shfl_up_sync(FULL, x.w[I], L);
}

struct Tile {
  long long gtile;   /* global tile id                                   */
  long long first;   /* global id of the first tile of this input        */
  long long last;    /* global id of the first tile of the next input    */
  long long base;    /* input word index of lane 0 word 0 (may be < 0)   */
  long long n;       /* characters in the input                          */
  long long W;       /* words in the input                               */
  unsigned long long epoch;
  int input;
  int lane;
  S vm;              /* per word: all ones if the word index is >= 0     */
  S em;              /* per word: the bits of positions before the input end */
  bool edge;         /* the tile has words before the input start or reaches its last word */
  unsigned int claim_g;      /* next_tile: the last tile handed out of the current claim  */
  int claim_left;            /* next_tile: tiles of the current claim not yet handed out  */
  unsigned long long *cnt_s; /* the warp's match counts of `input` per output, in shared memory
                                (added to counts when the input changes and at the end), or NULL */
  uint32_t pcin[NPRE_WORDS]; /* bit k: carry entering pre-pass addition k (warp-uniform)   */
};

/* Advance(x, N): marks move N positions forward; words before the input start read as 0. */
template <int N>
__device__ __forceinline__ S adv(const S &xin, const Tile &t) {
  constexpr int Q = N / 32, R = N % 32;
  const S x = xin & t.vm;
  S r;
#pragma unroll
  for (int j = 0; j < WPT; ++j) {
    const uint32_t cur = word_back(x, j - Q);
    if (R == 0) {
      r.w[j] = cur;
    } else {
      const uint32_t prev = word_back(x, j - Q - 1);
      r.w[j] = __funnelshift_r(cur, prev, R);
    }
  }
  return r;
}

__device__ __forceinline__ unsigned long long ld_relaxed(const unsigned long long *p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed(unsigned long long *p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

/* Rows of 32 tiles: the unit of the pre-pass bitmaps (see load_pre_carries). */
__device__ __forceinline__ long long pre_rows(const BgParams &p) { return (p.n_tiles + 31) >> 5; }

/* record = epoch << 4 | flag << 2 | P << 1 | G ; flag 1 = aggregate, 2 = inclusive carry */
__device__ __forceinline__ void publish(const BgParams &p, const Tile &t, int k, uint32_t flag,
                                        uint32_t P, uint32_t G) {
  if (t.lane == 0) {
    unsigned long long r = (t.epoch << 4) | ((unsigned long long)flag << 2) |
                           ((unsigned long long)P << 1) | (unsigned long long)G;
    st_relaxed(p.records + (long long)k * p.n_tiles + t.gtile, r);
  }
}

/* Bounded wait for a look-back record; returns an inclusive zero carry on timeout.
 * Lane 0 polls and broadcasts, so every lane takes the same path.  The wait ends when the
 * record carries this launch's epoch, after spin_limit clock64 cycles or 2^22 polls, or at once
 * when an earlier wait of this launch already timed out (so one lost record cannot make every
 * later tile wait its full budget). */
__device__ __forceinline__ unsigned long long wait_record(const unsigned long long *addr,
                                                          unsigned long long epoch,
                                                          long long spin_limit, uint32_t *state,
                                                          int lane) {
  unsigned long long r = 0;
  if (lane == 0) {
    const long long t0 = clock64();
    unsigned ns = 32;
    for (unsigned it = 0;; ++it) {
      r = ld_relaxed(addr);
      if ((r >> 4) == epoch) break;
      const bool aborted = (*(volatile uint32_t *)(state + 1) & BG_DEV_ERR_TIMEOUT) != 0u;
      if (aborted || it >= (1u << 22) || clock64() - t0 > spin_limit) {
        atomicOr(state + 1, BG_DEV_ERR_TIMEOUT);
        r = (epoch << 4) | (2ull << 2);
        break;
      }
      __nanosleep(ns);
      if (ns < 1024) ns <<= 1;
    }
  }
  return __shfl_sync(FULL, r, 0);
}

/* Carry entering tile `gtile`'s look-back lane for the addition whose records start at `rec`:
 * decoupled look-back, LBK * 32 predecessor records per step (lane l reads tiles
 * gtile-1-l*LBK .. gtile-(l+1)*LBK, nearest first).  A record "terminates" the walk when it fixes
 * the carry by itself: an inclusive carry, or an aggregate that generates a carry or does not
 * propagate one.  Every record before the nearest terminator is an aggregate that propagates and
 * does not generate, so the carry is simply the terminator's bit.  Control flow is warp-uniform
 * (decisions come from ballots / lane 0).  Waits are bounded like wait_record. */
#if BG_LOOKBACK_INLINE
static __device__ __forceinline__
#else
static __device__ __noinline__
#endif
uint32_t lookback(const unsigned long long *rec, long long gtile, long long first,
                  unsigned long long epoch, long long spin_limit, uint32_t *state, int lane) {
  constexpr int LBK = BG_LBK;
  long long base = gtile - 1;
  long long t0 = clock64();
  unsigned ns = 0, polls = 0;
  for (;;) {
    int term = LBK;        /* index of my nearest terminator, LBK = none                    */
    bool blocked = false;  /* an unpublished record comes before my nearest terminator      */
    uint32_t tG = 0u;
    bool before_input = false;
#pragma unroll
    for (int i = 0; i < LBK; ++i) {
      const long long j = base - (long long)lane * LBK - i;
      unsigned long long r;
      bool valid = true;
      if (j >= first) {
        r = ld_relaxed(rec + j);
        valid = (r >> 4) == epoch;
      } else {
        r = (epoch << 4) | (2ull << 2); /* before the input: carry 0 */
      }
      if (term == LBK && !blocked) {
        if (!valid) {
          blocked = true;
        } else {
          const uint32_t flag = (uint32_t)(r >> 2) & 3u;
          const uint32_t G = (uint32_t)r & 1u, P = (uint32_t)(r >> 1) & 1u;
          if (flag == 2u || (flag == 1u && (P == 0u || G == 1u))) {
            term = i;
            tG = G;
            before_input = j < first;
          }
        }
      }
    }
    const uint32_t tmask = __ballot_sync(FULL, term < LBK);
    const uint32_t bmask = __ballot_sync(FULL, blocked);
    const uint32_t stop = tmask | bmask;
    if (stop == 0u) { /* 32 * LBK propagating aggregates: keep walking */
      base -= 32 * LBK;
      t0 = clock64();
      polls = 0;
      ns = 0;
      continue;
    }
    const int l0 = __ffs(stop) - 1;
    if ((tmask >> l0) & 1u) {
      const uint32_t bi = __shfl_sync(FULL, before_input ? 1u : 0u, l0);
      if (bi && lane == 0) atomicOr(state + 1, BG_DEV_ERR_CHAIN);
      return __shfl_sync(FULL, tG, l0);
    }
    /* a record before the nearest terminator is not published yet: wait, bounded */
    long long el = clock64() - t0;
    el = __shfl_sync(FULL, el, 0);
    const uint32_t ab = __shfl_sync(FULL, *(volatile uint32_t *)(state + 1), 0);
    if ((ab & BG_DEV_ERR_TIMEOUT) || ++polls >= (1u << 22) || el > spin_limit) {
      if (lane == 0) atomicOr(state + 1, BG_DEV_ERR_TIMEOUT);
      return 0u;
    }
    if (polls > BG_LB_SPIN) {
      __nanosleep(ns);
      ns = ns ? (ns < 1024 ? ns * 2 : ns) : 64;
    }
  }
}

/* What an addition needs to know about its tile (passed by value to the out-of-line path). */
struct Lk {
  long long gtile, first;
  unsigned long long epoch;
  S vm;
};

/* Carry vector for addition k: bit l = carry entering lane l.  Gm/Pm are the lanes that
 * generate / propagate a carry; lanes below DL are ignored and the carry enters at DL. */
template <int DL>
__device__ __forceinline__ uint32_t carries(const BgParams &p, const Lk &L, int k, uint32_t Gm,
                                            uint32_t Pm) {
  static_assert(DL >= 0 && DL < HL || (HL == 0 && DL == 0), "carry lane must be in the halo");
  constexpr int OUTL = SL + DL; /* the successor tile's carry lane, in our coordinates */
  const int lane = threadIdx.x & 31;
  const uint32_t keep = ~((1u << DL) - 1u);
  Gm &= keep;
  Pm &= keep;
  const uint32_t A = Gm | Pm, B = Gm;
  uint32_t cin = 0;
  const bool own = (HL > 0) && ((Pm >> DL) & 1u);
  const bool succ = (HL > 0) && ((Pm >> (OUTL & 31)) & 1u);
  unsigned long long *rec = p.records + (long long)k * p.n_tiles;
  if (own) {
    if (succ) {
      const uint32_t c0 = (uint32_t)((unsigned long long)A + B) ^ A ^ B;
      const uint32_t span = (SL >= 32) ? FULL : ((1u << SL) - 1u);
      const uint32_t Pagg = (((Pm >> DL) & span) == span) ? 1u : 0u;
      if (lane == 0) st_relaxed(rec + L.gtile, (L.epoch << 4) | (1ull << 2) | ((unsigned long long)Pagg << 1) | ((c0 >> OUTL) & 1u));
    }
    cin = lookback(rec, L.gtile, L.first, L.epoch, p.spin_limit, p.state, lane);
  }
  const uint32_t cvec =
      (uint32_t)((unsigned long long)A + B + ((unsigned long long)cin << DL)) ^ A ^ B;
  if (succ && lane == 0) st_relaxed(rec + L.gtile, (L.epoch << 4) | (2ull << 2) | ((cvec >> OUTL) & 1u));
  return cvec;
}

/* Exact X + Y over the tile (positions ascend with bit significance after __brev). */
template <int DL>
__device__ __forceinline__ S add_carry(const BgParams &p, const Lk &L, int k, const S &X,
                                       const S &Y) {
  const int lane = threadIdx.x & 31;
  uint32_t xb[WPT], yb[WPT];
  uint32_t G = 0u, P = 1u;
#pragma unroll
  for (int j = 0; j < WPT; ++j) {
    xb[j] = __brev(X.w[j] & L.vm.w[j]);
    yb[j] = __brev(Y.w[j] & L.vm.w[j]);
    const uint32_t s = xb[j] + yb[j];
    const uint32_t g = s < xb[j] ? 1u : 0u;
    const uint32_t pp = s == FULL ? 1u : 0u;
    G = g | (pp & G);
    P &= pp;
  }
  const uint32_t Gm = __ballot_sync(FULL, G), Pm = __ballot_sync(FULL, P);
  const uint32_t cvec = carries<DL>(p, L, k, Gm, Pm);
  uint32_t c = (cvec >> lane) & 1u;
  S r;
#pragma unroll
  for (int j = 0; j < WPT; ++j) {
    const unsigned long long s = (unsigned long long)xb[j] + yb[j] + c;
    r.w[j] = __brev((uint32_t)s);
    c = (uint32_t)(s >> 32);
  }
  return r;
}

/* Out-of-line part of MatchStar (mode 0) / ScanThru (mode 1): the general addition. */
template <int DL>
__device__ __noinline__ S add_slow(const BgParams &p, const Lk L, int k, int mode, const S M,
                                   const S C) {
  const S Cm = C & L.vm;
  const S X = mode == 0 ? (M & C) : M;
  const S sum = add_carry<DL>(p, L, k, X, C);
  return mode == 0 ? ((sum ^ Cm) | M) : (sum & ~C);
}

/* Inline fast path shared by MatchStar and ScanThru: when the marker is zero in the whole warp
 * and the carry lane does not propagate, no carry can enter and the result is zero; the
 * successor's carry (zero) is published if it will be needed. */
template <int DL, bool E = true>
__device__ __forceinline__ bool add_is_zero(const BgParams &p, const Tile &t, int k, const S &M,
                                            const S &C) {
  uint32_t mo = 0u, ao = 1u;
#pragma unroll
  for (int j = 0; j < WPT; ++j) {
    mo |= M.w[j];
    ao &= ((C.w[j] & (E ? t.vm.w[j] : FULL)) == FULL) ? 1u : 0u;
  }
  if (__any_sync(FULL, mo != 0u)) return false;
  const uint32_t Pm = __ballot_sync(FULL, ao);
  if ((Pm >> DL) & 1u) return false;
  if ((Pm >> ((SL + DL) & 31)) & 1u) {
    if (t.lane == 0)
      st_relaxed(p.records + (long long)k * p.n_tiles + t.gtile, (t.epoch << 4) | (2ull << 2));
  }
  return true;
}

/* MatchStar(M, C) = (((M & C) + C) ^ C) | M   (bitgen/template/template_torch.py:392-407) */
template <int DL>
__device__ __forceinline__ S matchstar(const BgParams &p, const Tile &t, int k, const S &M,
                                       const S &C) {
  if (add_is_zero<DL>(p, t, k, M, C)) return zero();
  return add_slow<DL>(p, Lk{t.gtile, t.first, t.epoch, t.vm}, k, 0, M, C);
}

/* ScanThru(M, C) = (M + C) & ~C   (bitgen/template/template_torch.py:377-389) */
template <int DL>
__device__ __forceinline__ S scanthru(const BgParams &p, const Tile &t, int k, const S &M,
                                      const S &C) {
  if (add_is_zero<DL>(p, t, k, M, C)) return zero();
  return add_slow<DL>(p, Lk{t.gtile, t.first, t.epoch, t.vm}, k, 1, M, C);
}

/* Split form of an addition, so that the wait for a predecessor's carry overlaps other work:
 * add_begin computes the lanes' generate/propagate masks and publishes this tile's aggregate
 * right away (or, when the carry lane does not propagate, resolves everything locally);
 * add_end, issued later, runs the look-back if one is needed and forms the result. */
struct AddState {
  uint32_t xb[WPT], yb[WPT];
  uint32_t Gm, Pm, cvec;
  uint32_t state; /* 0 = look-back pending, 1 = result is zero, 2 = carries resolved */
};

template <int DL, bool E = true>
__device__ __forceinline__ AddState add_begin(const BgParams &p, const Tile &t, int k, int mode,
                                              const S &M, const S &C) {
  AddState a;
  a.Gm = a.Pm = a.cvec = 0u;
  if (add_is_zero<DL, E>(p, t, k, M, C)) {
    a.state = 1u;
#pragma unroll
    for (int j = 0; j < WPT; ++j) a.xb[j] = a.yb[j] = 0u;
    return a;
  }
  uint32_t G = 0u, P = 1u;
#pragma unroll
  for (int j = 0; j < WPT; ++j) {
    const uint32_t x = mode == 0 ? (M.w[j] & C.w[j]) : M.w[j];
    a.xb[j] = __brev(E ? (x & t.vm.w[j]) : x);
    a.yb[j] = __brev(E ? (C.w[j] & t.vm.w[j]) : C.w[j]);
    const uint32_t s = a.xb[j] + a.yb[j];
    const uint32_t g = s < a.xb[j] ? 1u : 0u;
    const uint32_t pp = s == FULL ? 1u : 0u;
    G = g | (pp & G);
    P &= pp;
  }
  constexpr int OUTL = SL + DL;
  const uint32_t keep = ~((1u << DL) - 1u);
  a.Gm = __ballot_sync(FULL, G) & keep;
  a.Pm = __ballot_sync(FULL, P) & keep;
  const uint32_t A = a.Gm | a.Pm, B = a.Gm;
  const bool own = (a.Pm >> DL) & 1u;
  const bool succ = (a.Pm >> (OUTL & 31)) & 1u;
  unsigned long long *rec = p.records + (long long)k * p.n_tiles;
  if (own) {
    if (succ && t.lane == 0) {
      const uint32_t c0 = (uint32_t)((unsigned long long)A + B) ^ A ^ B;
      const uint32_t span = (SL >= 32) ? FULL : ((1u << SL) - 1u);
      const uint32_t Pagg = (((a.Pm >> DL) & span) == span) ? 1u : 0u;
      st_relaxed(rec + t.gtile, (t.epoch << 4) | (1ull << 2) | ((unsigned long long)Pagg << 1) |
                                    ((c0 >> OUTL) & 1u));
    }
    a.state = 0u;
  } else {
    a.cvec = (uint32_t)((unsigned long long)A + B) ^ A ^ B;
    if (succ && t.lane == 0)
      st_relaxed(rec + t.gtile, (t.epoch << 4) | (2ull << 2) | ((a.cvec >> OUTL) & 1u));
    a.state = 2u;
  }
  return a;
}

template <int DL, bool E = true>
__device__ __forceinline__ S add_end(const BgParams &p, const Tile &t, int k, int mode,
                                     const AddState &a, const S &M, const S &C) {
  if (a.state == 1u) return zero();
  uint32_t cvec = a.cvec;
  if (a.state == 0u) {
    constexpr int OUTL = SL + DL;
    unsigned long long *rec = p.records + (long long)k * p.n_tiles;
    const uint32_t cin = lookback(rec, t.gtile, t.first, t.epoch, p.spin_limit, p.state, t.lane);
    const uint32_t A = a.Gm | a.Pm, B = a.Gm;
    cvec = (uint32_t)((unsigned long long)A + B + ((unsigned long long)cin << DL)) ^ A ^ B;
    if (((a.Pm >> (OUTL & 31)) & 1u) && t.lane == 0)
      st_relaxed(rec + t.gtile, (t.epoch << 4) | (2ull << 2) | ((cvec >> OUTL) & 1u));
  }
  uint32_t c = (cvec >> t.lane) & 1u;
  S r;
#pragma unroll
  for (int j = 0; j < WPT; ++j) {
    const unsigned long long s = (unsigned long long)a.xb[j] + a.yb[j] + c;
    const uint32_t sum = __brev((uint32_t)s);
    c = (uint32_t)(s >> 32);
    r.w[j] = mode == 0 ? ((sum ^ (E ? (C.w[j] & t.vm.w[j]) : C.w[j])) | M.w[j]) : (sum & ~C.w[j]);
  }
  return r;
}

/* Lane generate / propagate masks of X + Y for addition k's operands (lanes below DL cleared):
 * the part of add_begin that the pre-pass and add_known share. */
template <int DL, bool E>
__device__ __forceinline__ void add_masks(const Tile &t, int mode, const S &M, const S &C,
                                          uint32_t xb[WPT], uint32_t yb[WPT], uint32_t &Gm,
                                          uint32_t &Pm) {
  uint32_t G = 0u, P = 1u;
#pragma unroll
  for (int j = 0; j < WPT; ++j) {
    const uint32_t x = mode == 0 ? (M.w[j] & C.w[j]) : M.w[j];
    xb[j] = __brev(E ? (x & t.vm.w[j]) : x);
    yb[j] = __brev(E ? (C.w[j] & t.vm.w[j]) : C.w[j]);
    const uint32_t s = xb[j] + yb[j];
    const uint32_t g = s < xb[j] ? 1u : 0u;
    const uint32_t pp = s == FULL ? 1u : 0u;
    G = g | (pp & G);
    P &= pp;
  }
  const uint32_t keep = ~((1u << DL) - 1u);
  Gm = __ballot_sync(FULL, G) & keep;
  Pm = __ballot_sync(FULL, P) & keep;
}

/* Pre-pass: this tile's (generate, propagate) aggregate of an addition over its own lanes
 * [DL, SL + DL), computed with a zero carry entering lane DL (warp-uniform bits). */
template <int DL, bool E = true>
__device__ __forceinline__ void pre_aggregate(const Tile &t, int mode, const S &M, const S &C,
                                              uint32_t &G, uint32_t &P) {
  uint32_t xb[WPT], yb[WPT], Gm, Pm;
  add_masks<DL, E>(t, mode, M, C, xb, yb, Gm, Pm);
  constexpr int OUTL = SL + DL;
  const uint32_t A = Gm | Pm, B = Gm;
  const uint32_t c0 = (uint32_t)((unsigned long long)A + B) ^ A ^ B;
  const uint32_t span = (SL >= 32) ? FULL : ((1u << SL) - 1u);
  P = (((Pm >> DL) & span) == span) ? 1u : 0u;
  G = (c0 >> OUTL) & 1u;
}

/* pre_aggregate for a tile where the marker is known to be zero: nothing is generated, and the
 * tile propagates a carry exactly when the class is all ones over its own lanes.  `ones` is
 * ones_lanes() of the class. */
template <int DL>
__device__ __forceinline__ uint32_t pre_propagates(uint32_t ones) {
  const uint32_t span = (SL >= 32) ? FULL : ((1u << SL) - 1u);
  return ((ones >> DL) & span) == span ? 1u : 0u;
}

/* After tile l of a chunk of 32: move the tile's aggregate bits (bit k of pg / pp = addition k)
 * into the chunk words that lane k keeps for addition k. */
__device__ __forceinline__ void pre_collect(const uint32_t pg[NPRE_WORDS], const uint32_t pp[NPRE_WORDS],
                                            uint32_t gw[NPRE_WORDS], uint32_t pw[NPRE_WORDS],
                                            int l, int lane) {
#pragma unroll
  for (int j = 0; j < NPRE_WORDS; ++j) {
    gw[j] |= ((pg[j] >> lane) & 1u) << l;
    pw[j] |= ((pp[j] >> lane) & 1u) << l;
  }
}

/* End of a chunk of row `row` (tiles 32 row .. 32 row + 31): store the row words of every
 * pre-pass addition; a chunk shorter than the row ORs its tiles' bits into words the launch
 * zeroed. */
__device__ __forceinline__ void pre_flush(const BgParams &p, long long row,
                                          const uint32_t gw[NPRE_WORDS],
                                          const uint32_t pw[NPRE_WORDS], int lane, bool partial) {
  const long long R = pre_rows(p);
#pragma unroll
  for (int j = 0; j < NPRE_WORDS; ++j) {
    const int k = 32 * j + lane;
    if (k < NPRE) {
      uint32_t *b = p.pre_bits + 3 * R * k;
      if (!partial) {
        b[row] = gw[j];
        b[R + row] = pw[j];
      } else {
        if (gw[j]) atomicOr(b + row, gw[j]);
        if (pw[j]) atomicOr(b + R + row, pw[j]);
      }
    }
  }
}

/* Main pass for a pre-pass addition: the carry entering lane DL is known (t.pcin), so the
 * addition resolves without publishing or waiting.  Its result is formed by add_end. */
template <int DL, bool E = true>
__device__ __forceinline__ AddState add_known(const BgParams &p, const Tile &t, int k, int mode,
                                              const S &M, const S &C) {
  AddState a;
  const uint32_t cin = (t.pcin[k >> 5] >> (k & 31)) & 1u;
  uint32_t mo = 0u;
#pragma unroll
  for (int j = 0; j < WPT; ++j) mo |= M.w[j];
  if (cin == 0u && !__any_sync(FULL, mo != 0u)) {
    /* no marker and no carry: the sum is C itself, so the result is zero */
    a.state = 1u;
    a.Gm = a.Pm = a.cvec = 0u;
#pragma unroll
    for (int j = 0; j < WPT; ++j) a.xb[j] = a.yb[j] = 0u;
    return a;
  }
  add_masks<DL, E>(t, mode, M, C, a.xb, a.yb, a.Gm, a.Pm);
  const uint32_t A = a.Gm | a.Pm, B = a.Gm;
  a.cvec = (uint32_t)((unsigned long long)A + B + ((unsigned long long)cin << DL)) ^ A ^ B;
  a.state = 2u;
  return a;
}

/* ---------------------------------------------------------------------------------------
 * Tile scheduling, loads and stores
 * --------------------------------------------------------------------------------------- */
__device__ __forceinline__ void init(const BgParams &p, Tile &t) {
  t.lane = threadIdx.x & 31;
  t.input = 0;
  t.first = t.last = 0;   /* no input held yet */
  t.cnt_s = nullptr;
  t.claim_g = 0u;
  t.claim_left = 0;
  t.epoch = *(volatile const unsigned long long *)(p.state + 2);
}

/* Compact pre-pass data.  For pre-pass addition k, p.pre_bits + 3 * R * k (R = rows of 32 tiles)
 * holds three bitmaps of R words, bit l of word r standing for tile 32r + l: the tile generates
 * a carry [0, R), the tile propagates one [R, 2R), a carry enters the tile [2R, 3R).  The first
 * two are written by the pass that computes the aggregates, the third by the carry scan. */
/* Carries entering this tile for the pre-pass additions (warp-uniform bit k per addition). */
__device__ __forceinline__ void load_pre_carries(const BgParams &p, Tile &t) {
  const long long R = pre_rows(p);
#pragma unroll
  for (int w = 0; w < NPRE_WORDS; ++w) {
    const int k = w * 32 + t.lane;
    uint32_t c = 0u;
    if (NPRE > 0 && k < NPRE)
      c = (__ldg(p.pre_bits + 3 * R * k + 2 * R + (t.gtile >> 5)) >> (t.gtile & 31)) & 1u;
    t.pcin[w] = __ballot_sync(FULL, c != 0u);
  }
}

/* Fill `t` for global tile g.  `carries`: read the pre-pass carries (false in the passes that
 * run before the carry scan); `debug_wait`: take part in the wait-limit test (exactly one pass
 * over every tile does). */
#ifndef BG_WCOUNT
#define BG_WCOUNT 0
#endif
/* Match counts kept per warp (BG_WCOUNT outputs): counts[o][input] gets one atomic add per
 * output and input a warp worked on, instead of one per tile and output (the counts of all
 * outputs share a few cache lines, whose atomics would queue). */
__device__ __forceinline__ void count_cache_begin(Tile &t, unsigned long long *slots) {
  t.cnt_s = slots;
  for (int o = t.lane; o < BG_WCOUNT; o += 32) slots[o] = 0ull;
  __syncwarp();
}
__device__ __forceinline__ void flush_counts(const BgParams &p, const Tile &t) {
  if (BG_WCOUNT == 0 || t.cnt_s == nullptr) return;
  __syncwarp();
  for (int o = t.lane; o < BG_WCOUNT; o += 32) {
    const unsigned long long c = t.cnt_s[o];
    if (c) {
      if (p.counts) atomicAdd(p.counts + (long long)o * p.n_inputs + t.input, c);
      t.cnt_s[o] = 0ull;
    }
  }
  __syncwarp();
}

__device__ __forceinline__ void setup_tile(const BgParams &p, Tile &t, unsigned int g,
                                           bool carries = true, bool debug_wait = true) {
  /* find i: prefix[i] <= g < prefix[i+1]; a warp's tiles mostly stay in the input of its
   * previous tile, whose bounds and length the tile holds (no loads then) */
  if (!((long long)g >= t.first && (long long)g < t.last)) {
    flush_counts(p, t);   /* the counts gathered for the previous input */
    int lo = 0, hi = p.n_inputs;
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (p.tile_prefix[mid] <= (long long)g) lo = mid; else hi = mid;
    }
    t.input = lo;
    t.first = p.tile_prefix[lo];
    t.last = p.tile_prefix[lo + 1];
    t.n = p.in_len[lo];
    t.W = (t.n + 31) >> 5;
  }
  t.gtile = g;
  t.base = ((long long)g - t.first) * SW - (long long)HL * WPT;
#pragma unroll
  for (int j = 0; j < WPT; ++j) {
    const long long w = t.base + t.lane * WPT + j;
    t.vm.w[j] = (w >= 0) ? FULL : 0u;
    const long long rem = t.n - 32 * w;
    t.em.w[j] = rem >= 32 ? FULL : (rem <= 0 ? 0u : (FULL << (32 - rem)));
  }
  t.edge = t.base < 0 || t.base + 32 * WPT >= t.W;
  if (NPRE > 0 && carries) load_pre_carries(p, t);
  if (debug_wait && (long long)g == p.debug_wait_tile) /* wait-limit test: nobody writes this record */
    (void)wait_record(reinterpret_cast<const unsigned long long *>(p.state + 4), t.epoch,
                      p.spin_limit, p.state, t.lane);
}

/* setup_tile for tile g of a known input (first tile `first`, n bytes), from values the caller
 * holds: no table lookups (the classify pass walks a chunk of one input). */
__device__ __forceinline__ void setup_tile_in(const BgParams &p, Tile &t, unsigned int g,
                                              int input, long long first, long long n) {
  t.input = input;
  t.gtile = g;
  t.first = first;
  t.last = first;     /* the next setup_tile looks its input up */
  t.n = n;
  t.W = (n + 31) >> 5;
  t.base = ((long long)g - first) * SW - (long long)HL * WPT;
#pragma unroll
  for (int j = 0; j < WPT; ++j) {
    const long long w = t.base + t.lane * WPT + j;
    t.vm.w[j] = (w >= 0) ? FULL : 0u;
    const long long rem = n - 32 * w;
    t.em.w[j] = rem >= 32 ? FULL : (rem <= 0 ? 0u : (FULL << (32 - rem)));
  }
  t.edge = t.base < 0 || t.base + 32 * WPT >= t.W;
  if ((long long)g == p.debug_wait_tile) /* wait-limit test: nobody writes this record */
    (void)wait_record(reinterpret_cast<const unsigned long long *>(p.state + 4), t.epoch,
                      p.spin_limit, p.state, t.lane);
}

/* Claim the next tile (tiles are handed out in increasing order, which is what makes the
 * look-back deadlock free: a tile only waits for tiles claimed before it). */
#ifndef BG_CLAIM_TILES
#define BG_CLAIM_TILES 1
#endif
__device__ __forceinline__ bool next_tile(const BgParams &p, Tile &t) {
  /* BG_CLAIM_TILES consecutive tiles per claim (fewer atomics on the one counter); the warp
   * runs them in order, so every tile still waits only for tiles claimed before it */
  unsigned int g = 0;
  if (BG_CLAIM_TILES > 1 && t.claim_left > 0) {
    g = ++t.claim_g;
    --t.claim_left;
  } else {
    if (t.lane == 0) g = atomicAdd(p.state, (unsigned int)BG_CLAIM_TILES);
    g = __shfl_sync(FULL, g, 0);
    t.claim_g = g;
    t.claim_left = BG_CLAIM_TILES - 1;
  }
  if ((long long)g >= p.n_tiles) return false;
  setup_tile(p, t, g);
  return true;
}

/* Block-wide claim of one tile per warp (lockstep form: the warps of a block run the same part
 * functions between barriers).  Returns the block's first tile; all threads must call it. */
__device__ __forceinline__ unsigned int claim_block(const BgParams &p, unsigned int *slot) {
  __syncthreads();
  if (threadIdx.x == 0) *slot = atomicAdd(p.state, blockDim.x >> 5);
  __syncthreads();
  return *slot;
}

/* The 32 bytes of word (lane * WPT + j) of the tile as eight little-endian 32-bit words;
 * bytes before the input start or at or beyond its end read as zero. */
__device__ __forceinline__ void load_word_bytes(const BgParams &p, const Tile &t, int j,
                                                uint32_t u[8]) {
  const uint8_t *src = p.in_bytes + p.in_off[t.input];
  const long long w = t.base + t.lane * WPT + j;
  if (w >= 0 && 32 * w + 32 <= t.n) {
    const uint4 *q = reinterpret_cast<const uint4 *>(src + 32 * w);
    const uint4 a = __ldg(q), c = __ldg(q + 1);
    u[0] = a.x; u[1] = a.y; u[2] = a.z; u[3] = a.w;
    u[4] = c.x; u[5] = c.y; u[6] = c.z; u[7] = c.w;
  } else {
#pragma unroll
    for (int q = 0; q < 8; ++q) u[q] = 0u;
    if (w >= 0 && w < t.W) {
      /* the input's last, partial word: its bytes one by one (static indices keep u in
         registers) */
      const long long rem = t.n - 32 * w;
#pragma unroll
      for (int k = 0; k < 32; ++k)
        if (k < rem) u[k >> 2] |= (uint32_t)__ldg(src + 32 * w + k) << (8 * (k & 3));
    }
  }
}

/* load_word_bytes for the tile `delta` words after t in the same input (the classify pass's
 * prefetch of its next tile: a chunk inside one input walks consecutive tiles). */
__device__ __forceinline__ void load_word_bytes_ahead(const BgParams &p, const Tile &t,
                                                      long long delta, int j, uint32_t u[8]) {
  const uint8_t *src = p.in_bytes + p.in_off[t.input];
  const long long w = t.base + delta + t.lane * WPT + j;
  if (w >= 0 && 32 * w + 32 <= t.n) {
    const uint4 *q = reinterpret_cast<const uint4 *>(src + 32 * w);
    const uint4 a = __ldg(q), c = __ldg(q + 1);
    u[0] = a.x; u[1] = a.y; u[2] = a.z; u[3] = a.w;
    u[4] = c.x; u[5] = c.y; u[6] = c.z; u[7] = c.w;
  } else {
#pragma unroll
    for (int q = 0; q < 8; ++q) u[q] = 0u;
    if (w >= 0 && w < t.W) {
      /* the input's last, partial word: its bytes one by one (static indices keep u in
         registers) */
      const long long rem = t.n - 32 * w;
#pragma unroll
      for (int k = 0; k < 32; ++k)
        if (k < rem) u[k >> 2] |= (uint32_t)__ldg(src + 32 * w + k) << (8 * (k & 3));
    }
  }
}

__device__ __forceinline__ void load_basis(const BgParams &p, const Tile &t, S b[8]) {
  if (p.input_kind == BG_INPUT_BASIS) {
    const uint32_t *src = p.in_basis + p.in_off[t.input];
#pragma unroll
    for (int j = 0; j < WPT; ++j) {
      const long long w = t.base + t.lane * WPT + j;
      const bool ok = w >= 0 && w < t.W;
#pragma unroll
      for (int i = 0; i < 8; ++i) b[i].w[j] = ok ? __ldg(src + i * p.basis_stride + w) : 0u;
    }
    return;
  }
#pragma unroll
  for (int j = 0; j < WPT; ++j) {
    uint32_t u[8];
    load_word_bytes(p, t, j, u);
    uint32_t o[8];
    transpose32(u, o);
#pragma unroll
    for (int i = 0; i < 8; ++i) b[i].w[j] = o[i];
  }
}

/* Count (and list as sparse positions) the bits of `vals`, this lane's exact words of output o
 * for this tile (bits at or beyond the input end already cleared). */
static __device__ __forceinline__ void store_new_bits(const BgParams &p, const Tile &t, int o,
                                                      const S &vals) {
  uint32_t cnt = 0;
#pragma unroll
  for (int j = 0; j < WPT; ++j) cnt += __popc(vals.w[j]);
  if (p.positions && __any_sync(FULL, cnt != 0u)) {
    /* sparse output: one slot range per warp, then each lane writes its own positions */
    uint32_t incl = cnt;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t y = __shfl_up_sync(FULL, incl, d);
      if (t.lane >= d) incl += y;
    }
    const uint32_t total = __shfl_sync(FULL, incl, 31);
    unsigned long long at = 0;
    if (t.lane == 31)
      at = atomicAdd(reinterpret_cast<unsigned long long *>(p.state + 6), (unsigned long long)total);
    at = __shfl_sync(FULL, at, 31) + (incl - cnt);
    const unsigned long long key =
        ((unsigned long long)o << 52) | ((unsigned long long)t.input << 32);
#pragma unroll
    for (int j = 0; j < WPT; ++j) {
      uint32_t val = vals.w[j];
      const long long w = t.base + t.lane * WPT + j;
      while (val) {
        const int b = 31 - __clz(val); /* highest set bit = lowest position */
        val &= ~(1u << b);
        if ((long long)at < p.pos_capacity)
          p.positions[at] = key | (unsigned long long)(32 * w + (31 - b));
        else
          atomicOr(p.state + 1, BG_DEV_ERR_CAPACITY);
        ++at;
      }
    }
  }
  if (p.counts) {
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) cnt += __shfl_xor_sync(FULL, cnt, d);
    if (t.lane == 0 && cnt) {
      if (BG_WCOUNT > 0 && t.cnt_s != nullptr && o < BG_WCOUNT) t.cnt_s[o] += cnt;
      else atomicAdd(p.counts + (long long)o * p.n_inputs + t.input, (unsigned long long)cnt);
    }
  }
}

/* Write output stream o for this tile (lanes >= HL, words inside the input; characters at or
 * beyond n are cleared) and add its popcount to counts[o][input]. */
static __device__ __noinline__ void store(const BgParams &p, const Tile &t, int o, const S v) {
  uint32_t *dst = p.out ? p.out + (long long)o * p.out_stride + p.out_off[t.input] : nullptr;
  S vals;
#pragma unroll
  for (int j = 0; j < WPT; ++j) {
    const long long w = t.base + t.lane * WPT + j;
    vals.w[j] = 0u;
    if (t.lane >= HL && t.lane < 32 - TL && w >= 0 && w < t.W) {
      uint32_t val = v.w[j];
      const long long rem = t.n - 32 * w;
      if (rem < 32) val &= FULL << (32 - rem);
      if (dst) dst[w] = val;
      vals.w[j] = val;
    }
  }
  store_new_bits(p, t, o, vals);
}

#if BG_PREFILTER
/* Q-gram prefilter (tables generated by bitgen_gb300/prefilter.py).  The q-grams (BG_QGRAM = 3
 * or 4 bytes) ending at every BG_STRIDE-th byte of the bytes this warp computes (byte e of a
 * 32-byte lane word with e % BG_STRIDE == BG_STRIDE - 1) are probed in the Bloom bitmap `bloom`
 * (2^BG_BLOOM_BITS bits, shared memory); a hit is resolved in the exact open-addressed table
 * (also in shared memory), whose records set bits of the tile's run mask.  A q-gram key holds
 * its oldest byte in bits 0-7; bytes before the warp's first byte read as zero. */
#ifndef BG_QGRAM
#define BG_QGRAM 3
#endif
#ifndef BG_STRIDE
#define BG_STRIDE 1
#endif
#ifndef BG_WILD
#define BG_WILD 0 /* bit 0 / 1: the exact table holds 4-grams with a free oldest / newest byte */
#endif
constexpr int QG = BG_QGRAM, QS = BG_STRIDE;
constexpr int NPROBE = 32 / QS;              /* probes per 32-byte lane word */
static_assert((QG == 3 || QG == 4) && (QS == 1 || QS == 2), "q-gram configuration");
constexpr uint32_t BLOOM_HASH = 0x9E3779B1u, EXACT_HASH = 0x85EBCA6Bu;

/* Exact lookup of a q-gram whose Bloom bit is set (all tables in shared memory).  `pre3` holds
 * the three bytes before the q-gram (the nearest in bits 0-7).  Slot s holds the key in keys[s]
 * and info[s] = start << 8 | count of its records (0 = empty slot); record i is
 * recs[2i] = bytes | n << 24 and recs[2i + 1] = the bit it sets when the n nearest bytes of
 * pre3 equal `bytes` (n = 0: always).  Bit b goes to run[(b / 32) * 32] (the tile's run words
 * in the warp's shared memory, 32 words apart). */
static __device__ __forceinline__ void qgram_exact(uint32_t key, uint32_t pre3, const uint32_t *keys,
                                                const uint32_t *info, const uint32_t *recs,
                                                int log2, uint32_t *run) {
  const uint32_t slots = 1u << log2;
  uint32_t s = (key * EXACT_HASH) >> (32 - log2);
  for (uint32_t it = 0; it < slots; ++it) {
    const uint32_t e = info[s];
    if (e == 0u) return;
    if (keys[s] == key) {
      for (uint32_t i = e >> 8, n = e & 255u; n > 0u; --n, ++i) {
        const uint32_t r = recs[2 * i], bit = recs[2 * i + 1];
        const uint32_t cmp = (1u << (8u * (r >> 24))) - 1u; /* n <= 3 */
        if (((pre3 ^ r) & cmp) == 0u && bit < 32u * BG_NRUN) atomicOr(run + (bit >> 5) * 32u, 1u << (bit & 31u));
      }
      return;
    }
    s = (s + 1u) & (slots - 1u);
  }
}

/* Bloom bit of q-gram x at bit 0 of the result (the other bits are arbitrary).  The word is the
 * top BG_BLOOM_BITS - 5 bits of the product x * BLOOM_HASH (for a trigram the constant is
 * shifted up by 8, which makes the product ignore the byte above the trigram); the bit within
 * the word is x's low 5 bits, the low bits of the oldest byte: a funnel shift in wrap mode
 * rotates the word right by exactly that. */
__device__ __forceinline__ uint32_t bloom_bit(uint32_t x, const uint32_t *bloom) {
  constexpr uint32_t M = QG == 3 ? (BLOOM_HASH << 8) : BLOOM_HASH;
  const uint32_t w = bloom[(x * M) >> (32 - BG_BLOOM_BITS + 5)];
  return __funnelshift_r(w, w, x);
}

/* The q-gram ending at byte e (0..31) of a lane word u[0..7] (little-endian 32-bit words),
 * with `pw` the previous lane word's last 32-bit word; bytes of a trigram key above bit 23 are
 * arbitrary. */
template <int E>
__device__ __forceinline__ uint32_t qgram_at(const uint32_t *u, uint32_t pw) {
  constexpr int I = E >> 2, R = E & 3;
  const uint32_t lo = I == 0 ? pw : u[I > 0 ? I - 1 : 0], hi = u[I];
  if (QG == 4) {
    if (R == 3) return hi;
    return __byte_perm(lo, hi, R == 0 ? 0x4321 : (R == 1 ? 0x5432 : 0x6543));
  }
  if (R == 2) return hi;
  if (R == 3) return hi >> 8;
  return __byte_perm(lo, hi, R == 0 ? 0x0432 : 0x0543);
}

/* Probes of one lane word: bit 32 - NPROBE + k of the result = the Bloom bit of probe k
 * (the q-gram ending at byte QS * k + QS - 1).  Each probe's bit enters at bit 31 while the
 * earlier ones move down one place. */
template <int K>
struct Probes {
  static __device__ __forceinline__ uint32_t run(const uint32_t *u, uint32_t pw,
                                                 const uint32_t *bloom, uint32_t acc) {
    acc = __funnelshift_r(acc, bloom_bit(qgram_at<QS * K + QS - 1>(u, pw), bloom), 1);
    return Probes<K + 1>::run(u, pw, bloom, acc);
  }
};
template <>
struct Probes<NPROBE> {
  static __device__ __forceinline__ uint32_t run(const uint32_t *, uint32_t, const uint32_t *,
                                                 uint32_t acc) {
    return acc;
  }
};

#ifndef BG_BASIS_FILTER
#define BG_BASIS_FILTER 0
#endif
#ifndef BG_HIT_CAP
#define BG_HIT_CAP 128 /* Bloom-hit records a warp holds per chunk */
#endif

/* A classify warp's state for one chunk of tiles (row `row`, tiles row * 32 + l): the filter
 * tables in shared memory, the chunk's run words (runs_s[w * 32 + l]: word w of tile l) and the
 * Bloom hits not yet looked up (hits_s, n_hits records).  A record is (tile l << 16 | lane word,
 * probe mask): the probes of that lane word whose Bloom bit was set. */
struct ClsCtx {
  const uint32_t *bloom, *keys, *info, *recs, *always;
  int log2;
  uint32_t *runs_s;
  uint2 *hits_s;
  uint32_t n_hits;
  long long row;
};

/* Byte `pos` of input `in` as the classify probes saw it: zero before the input, at or beyond
 * its end, and before the first byte `lo` of the warp that probed it. */
__device__ __forceinline__ uint32_t probe_byte(const BgParams &p, int in, long long n, long long lo,
                                               long long pos) {
  if (pos < lo || pos < 0 || pos >= n) return 0u;
  if (p.input_kind == BG_INPUT_BYTES) return __ldg(p.in_bytes + p.in_off[in] + pos);
  const uint32_t *src = p.in_basis + p.in_off[in] + (pos >> 5);
  const int sh = 31 - (int)(pos & 31);
  uint32_t b = 0u;
#pragma unroll
  for (int i = 0; i < 8; ++i) b |= ((__ldg(src + i * p.basis_stride) >> sh) & 1u) << (7 - i);
  return b;
}

/* Look up every recorded Bloom hit of the chunk, one record per lane (so a warp resolves up to
 * 32 hits in the time of one): the q-gram ending at the probed byte and the three bytes before
 * it, read again from the input, go through the exact table, whose records set run bits of the
 * hit's tile in runs_s.  Clears the records. */
__device__ __forceinline__ void resolve_hits(const BgParams &p, ClsCtx &c, int lane) {
  __syncwarp();
  for (uint32_t i = lane; i < c.n_hits; i += 32) {
    const uint2 rec = c.hits_s[i];
    const int l = (int)(rec.x >> 16), lw = (int)(rec.x & 0xffffu);
    const long long g = c.row * 32 + l;
    int lo = 0, hi = p.n_inputs; /* the tile's input */
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (p.tile_prefix[mid] <= g) lo = mid; else hi = mid;
    }
    const long long n = p.in_len[lo];
    const long long wbase = (g - p.tile_prefix[lo]) * SW - (long long)HL * WPT; /* warp's first word */
    for (uint32_t m = rec.y; m; m &= m - 1u) {
      const int k = __ffs(m) - 1 - (32 - NPROBE);
      const long long e = 32 * (wbase + lw) + QS * k + QS - 1; /* byte position in the input */
      uint32_t v[7];
#pragma unroll
      for (int d = 0; d < 7; ++d) v[d] = probe_byte(p, lo, n, 32 * wbase, e - d);
      const uint32_t key = QG == 4 ? (v[3] | v[2] << 8 | v[1] << 16 | v[0] << 24)
                                   : (v[2] | v[1] << 8 | v[0] << 16);
      const uint32_t pre3 = QG == 4 ? (v[4] | v[5] << 8 | v[6] << 16)
                                    : (v[3] | v[4] << 8 | v[5] << 16);
      qgram_exact(key, pre3, c.keys, c.info, c.recs, c.log2, c.runs_s + l);
      /* q-grams registered with a free oldest / newest byte are stored with that byte zeroed */
      if (BG_WILD & 1) qgram_exact(key & ~0xffu, pre3, c.keys, c.info, c.recs, c.log2, c.runs_s + l);
      if (BG_WILD & 2)
        qgram_exact(key & (QG == 4 ? 0x00ffffffu : 0x0000ffffu), pre3, c.keys, c.info, c.recs,
                    c.log2, c.runs_s + l);
    }
  }
  __syncwarp();
  c.n_hits = 0;
}

/* Load tile l's bytes into raw (lane word j = raw[j][0..7], little-endian), start its run words
 * in runs_s with the bits of the terms that always run, probe the q-grams and record the Bloom
 * hits (looked up later, by resolve_hits, for the whole chunk).  Inputs given as basis planes:
 * the bytes are rebuilt from the planes (bytes at or beyond the input's length are the planes'
 * padding there), and every term runs, or, with BG_BASIS_FILTER, the rebuilt bytes are
 * scanned the same way (the padding can only add hits).  The basis planes of the bytes, where
 * a caller needs them, come from basis_of. */
__device__ __forceinline__ void load_scan(const BgParams &p, Tile &t, uint32_t raw[WPT][8],
                                          ClsCtx &c, int l, bool have_bytes = false) {
  uint32_t *run = c.runs_s + l;
  if (have_bytes) {
    /* raw already holds the tile's bytes (prefetched by the caller) */
  } else if (p.input_kind == BG_INPUT_BASIS) {
    S b[8];
    load_basis(p, t, b);
#pragma unroll
    for (int j = 0; j < WPT; ++j) {
      uint32_t o[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) o[i] = b[i].w[j];
      untranspose32(o, raw[j]);
    }
    if (!BG_BASIS_FILTER) {
      for (int w = t.lane; w < BG_NRUN; w += 32) run[32 * w] = FULL;
      return;
    }
  } else {
#pragma unroll
    for (int j = 0; j < WPT; ++j) load_word_bytes(p, t, j, raw[j]);
  }
  /* every run word of the tile starts from the terms that always run (a lane per word, more
     than 32 words in turns) */
  for (int w = t.lane; w < BG_NRUN; w += 32) run[32 * w] = c.always[w];
  uint32_t prev = __shfl_up_sync(FULL, raw[WPT - 1][7], 1);
  if (t.lane == 0) prev = 0u;
  constexpr uint32_t KEEP = NPROBE == 32 ? FULL : ~((1u << (32 - NPROBE)) - 1u);
  uint32_t hits[WPT];
  uint32_t any = 0u;
#pragma unroll
  for (int j = 0; j < WPT; ++j) {
    hits[j] = Probes<0>::run(raw[j], prev, c.bloom, 0u) & KEEP;
    any |= hits[j];
    prev = raw[j][7];
  }
  if (__any_sync(FULL, any != 0u)) {
    uint32_t n = c.n_hits;
#pragma unroll
    for (int j = 0; j < WPT; ++j) {
      const uint32_t hb = __ballot_sync(FULL, hits[j] != 0u);
      n += __popc(hb);
    }
    if (n > BG_HIT_CAP) {
      /* more hits than the chunk's record buffer holds (text dense in filter keys): every
       * term runs on this tile, which is exact, and its hits need no lookup */
      for (int w = t.lane; w < BG_NRUN; w += 32) run[32 * w] = FULL;
      return;
    }
#pragma unroll
    for (int j = 0; j < WPT; ++j) {
      const uint32_t hb = __ballot_sync(FULL, hits[j] != 0u);
      if (hits[j])
        c.hits_s[c.n_hits + __popc(hb & ((1u << t.lane) - 1u))] =
            make_uint2(((uint32_t)l << 16) | (uint32_t)(t.lane * WPT + j), hits[j]);
      c.n_hits += __popc(hb);
    }
  }
}

/* The basis planes of the tile's bytes (as load_basis gives them). */
__device__ __forceinline__ void basis_of(const uint32_t raw[WPT][8], S b[8]) {
#pragma unroll
  for (int j = 0; j < WPT; ++j) {
    uint32_t o[8];
    transpose32(raw[j], o);
#pragma unroll
    for (int i = 0; i < 8; ++i) b[i].w[j] = o[i];
  }
}

/* Lanes whose bytes are all outside {X0, X1, X2} (the first K of them) and whose words lie
 * inside the input: ones_lanes of the class of the other bytes, from the bytes themselves.
 * A byte equals x exactly when the byte of v = w ^ (x * 0x01010101) is zero, and
 * (v - 0x01010101) & ~v & 0x80808080 is non-zero exactly when some byte of v is zero. */
template <int K, uint32_t X0, uint32_t X1 = 0u, uint32_t X2 = 0u>
__device__ __forceinline__ uint32_t excl_lanes(const Tile &t, const uint32_t raw[WPT][8]) {
  uint32_t h = 0u, in = 1u;
#pragma unroll
  for (int j = 0; j < WPT; ++j) {
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const uint32_t w = raw[j][i];
      const uint32_t v0 = w ^ (X0 * 0x01010101u);
      h |= (v0 - 0x01010101u) & ~v0 & 0x80808080u;
      if (K > 1) {
        const uint32_t v1 = w ^ (X1 * 0x01010101u);
        h |= (v1 - 0x01010101u) & ~v1 & 0x80808080u;
      }
      if (K > 2) {
        const uint32_t v2 = w ^ (X2 * 0x01010101u);
        h |= (v2 - 0x01010101u) & ~v2 & 0x80808080u;
      }
    }
    in &= t.vm.w[j] == FULL ? 1u : 0u;
  }
  return __ballot_sync(FULL, h == 0u && in);
}

/* Classes of the look-back carry obligations, for a cheap test before the exact one: bit c of
 * the result is set when the lane's first four bytes all lie in class c (tab[b] holds the
 * classes of byte b).  A lane whose words are all ones in class c has this bit set. */
__device__ __forceinline__ uint32_t first4_classes(const uint32_t raw[WPT][8], const uint32_t *tab) {
  const uint32_t w = raw[0][0];
  return tab[w & 255u] & tab[(w >> 8) & 255u] & tab[(w >> 16) & 255u] & tab[w >> 24];
}

/* Lanes whose words of class stream C are all ones (inside the input): an addition over C
 * with a zero marker can only take or pass on a carry through such lanes. */
__device__ __forceinline__ uint32_t ones_lanes(const Tile &t, const S &C) {
  uint32_t a = 1u;
#pragma unroll
  for (int j = 0; j < WPT; ++j) a &= ((C.w[j] & t.vm.w[j]) == FULL) ? 1u : 0u;
  return __ballot_sync(FULL, a);
}
#endif

#ifdef BG_NOUT
/* Per-warp output accumulators in shared memory, laid out [output][word][lane] so that a warp's
 * accesses are conflict free.  Only the owning warp touches its region. */
__device__ __forceinline__ void acc_clear(uint32_t *acc, const Tile &t) {
#pragma unroll 4
  for (int i = 0; i < BG_NOUT * WPT; ++i) acc[i * 32 + t.lane] = 0u;
}

__device__ __forceinline__ void acc_or(uint32_t *acc, int o, const S v) {
  const int lane = threadIdx.x & 31;
  uint32_t x = 0;
#pragma unroll
  for (int j = 0; j < WPT; ++j) x |= v.w[j];
  if (__any_sync(FULL, x != 0u)) {
#pragma unroll
    for (int j = 0; j < WPT; ++j) acc[(o * WPT + j) * 32 + lane] |= v.w[j];
  }
}

/* Split form: write zeros to output o's words of this tile (the words `store` would write),
 * for tiles on which the part computing o does not run. */
__device__ __forceinline__ void zero_store(const BgParams &p, const Tile &t, int o) {
  if (!p.out) return;
  uint32_t *dst = p.out + (long long)o * p.out_stride + p.out_off[t.input];
#pragma unroll
  for (int j = 0; j < WPT; ++j) {
    const long long w = t.base + t.lane * WPT + j;
    if (t.lane >= HL && t.lane < 32 - TL && w >= 0 && w < t.W) dst[w] = 0u;
  }
}

/* Launches without output streams (pos_set): insert position key `key` into the set; true when
 * it was not there yet.  Linear probing from a multiplicative hash; a full set (which the
 * runtime sizes at twice the position capacity) reports BG_DEV_ERR_SETFULL. */
__device__ __forceinline__ bool set_insert(const BgParams &p, unsigned long long key) {
  unsigned long long h = (key * 0x9E3779B97F4A7C15ull) >> 20;
  for (long long i = 0; i <= p.pos_set_mask; ++i) {
    const unsigned long long at = (h + (unsigned long long)i) & (unsigned long long)p.pos_set_mask;
    const unsigned long long prev = atomicCAS(p.pos_set + at, ~0ull, key);
    if (prev == ~0ull) return true;
    if (prev == key) return false;
  }
  atomicOr(p.state + 1, BG_DEV_ERR_SETFULL);
  return false;
}

/* merge_store for launches without output streams: the bits of this part's value of output o
 * that no part set before are those whose positions enter the set first; only they are
 * counted and listed. */
static __device__ __noinline__ void set_store(const BgParams &p, const Tile &t, int o, const S v) {
  S nb;
  const unsigned long long key = ((unsigned long long)o << 52) | ((unsigned long long)t.input << 32);
#pragma unroll
  for (int j = 0; j < WPT; ++j) {
    const long long w = t.base + t.lane * WPT + j;
    nb.w[j] = 0u;
    if (t.lane >= HL && t.lane < 32 - TL && w >= 0 && w < t.W) {
      uint32_t val = v.w[j];
      const long long rem = t.n - 32 * w;
      if (rem < 32) val &= FULL << (32 - rem);
      while (val) {
        const int b = 31 - __clz(val); /* highest set bit = lowest position */
        val &= ~(1u << b);
        if (set_insert(p, key | (unsigned long long)(32 * w + (31 - b)))) nb.w[j] |= 1u << b;
      }
    }
  }
  store_new_bits(p, t, o, nb);
}

/* Split form with outputs shared by several parts: OR this part's value of output o into the
 * tile's words (which the classify pass zeroed) and count, and list as positions, only the
 * bits it newly sets, so that counts stay exact whichever parts set a bit first.  Needs the
 * output streams (p.out). */
static __device__ __noinline__ void merge_store(const BgParams &p, const Tile &t, int o, const S v) {
  uint32_t x = 0u;
#pragma unroll
  for (int j = 0; j < WPT; ++j) x |= v.w[j];
  if (!__any_sync(FULL, x != 0u)) return;
  if (!p.out) {
    set_store(p, t, o, v);
    return;
  }
  uint32_t *dst = p.out + (long long)o * p.out_stride + p.out_off[t.input];
  S nb;
#pragma unroll
  for (int j = 0; j < WPT; ++j) {
    const long long w = t.base + t.lane * WPT + j;
    nb.w[j] = 0u;
    if (t.lane >= HL && t.lane < 32 - TL && w >= 0 && w < t.W) {
      uint32_t val = v.w[j];
      const long long rem = t.n - 32 * w;
      if (rem < 32) val &= FULL << (32 - rem);
      if (val) nb.w[j] = val & ~atomicOr(dst + w, val);
    }
  }
  store_new_bits(p, t, o, nb);
}

/* Split form with merged outputs: zero this tile's words of outputs 0..n-1 (the words `store`
 * would write), so that the parts can OR into them. */
__device__ __forceinline__ void zero_outputs(const BgParams &p, const Tile &t, int n) {
  if (!p.out) return;
  uint32_t *dst = p.out + p.out_off[t.input];
  bool ok[WPT];
#pragma unroll
  for (int j = 0; j < WPT; ++j) {
    const long long w = t.base + t.lane * WPT + j;
    ok[j] = t.lane >= HL && t.lane < 32 - TL && w >= 0 && w < t.W;
  }
  const long long w0 = t.base + t.lane * WPT;
  for (int o = 0; o < n; ++o, dst += p.out_stride) {
#pragma unroll
    for (int j = 0; j < WPT; ++j)
      if (ok[j]) dst[w0 + j] = 0u;
  }
}

/* Split form, classify: the launch's prologue, which the runtime's prologue kernel and counts
 * memset do for the other forms.  Block 0 clears the tile and match-position counters and
 * advances the launch epoch (only the execute pass reads it); all blocks clear the counts. */
__device__ __forceinline__ void cls_prologue(const BgParams &p, int n_out) {
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    p.state[0] = 0u;
    p.state[6] = 0u;
    p.state[7] = 0u;
    unsigned long long *ep = reinterpret_cast<unsigned long long *>(p.state + 2);
    *ep = *ep + 1ull;
  }
  if (p.counts) {
    const long long nc = (long long)n_out * p.n_inputs;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nc;
         i += (long long)gridDim.x * blockDim.x)
      p.counts[i] = 0ull;
  }
  if (p.pos_set) { /* an empty position set for the execute pass (slots: a multiple of 2) */
    ulonglong2 *s2 = reinterpret_cast<ulonglong2 *>(p.pos_set);
    const long long n2 = (p.pos_set_mask + 1) >> 1;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n2;
         i += (long long)gridDim.x * blockDim.x)
      s2[i] = make_ulonglong2(~0ull, ~0ull);
  }
}

/* Split form, classify: the input holding all of tiles g0 .. g1-1, or -1 when they span
 * several inputs. */
__device__ __forceinline__ int chunk_input(const BgParams &p, long long g0, long long g1) {
  int lo = 0, hi = p.n_inputs;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (p.tile_prefix[mid] <= g0) lo = mid; else hi = mid;
  }
  return p.tile_prefix[lo + 1] >= g1 ? lo : -1;
}

/* Zero words [lo, hi) of dst with the warp: scalar stores up to a 16-byte boundary, then
 * 16-byte stores, then the scalar tail. */
__device__ __forceinline__ void zero_span(uint32_t *dst, long long lo, long long hi, int lane) {
  if (hi <= lo) return;
  const unsigned mis = (unsigned)(((16u - ((unsigned)(unsigned long long)(dst + lo) & 15u)) & 15u) >> 2);
  const long long head = lo + mis < hi ? lo + mis : hi;
  if (lo + lane < head) dst[lo + lane] = 0u;
  const long long nv = (hi - head) >> 2;
  uint4 *v = reinterpret_cast<uint4 *>(dst + head);
  for (long long i = lane; i < nv; i += 32) v[i] = make_uint4(0u, 0u, 0u, 0u);
  const long long tail = head + 4 * nv;
  if (tail + lane < hi) dst[tail + lane] = 0u;
}

/* Zero words [lo, hi) of dst with bulk copies from `zbytes` bytes of zeros in shared memory
 * (shared-memory address zsm): the lanes store the few words up to a 16-byte boundary and after
 * the last one, lane 0 has the copy engine write the 16-byte aligned middle (cp.async.bulk:
 * both addresses 16-byte aligned, sizes multiples of 16), without load-store instructions of
 * its own.  The copies are committed as one bulk group; the kernel waits for its groups
 * (bulk_wait) before it exits. */
__device__ __forceinline__ void bulk_zero_span(uint32_t *dst, long long lo, long long hi, int lane,
                                               uint32_t zsm, uint32_t zbytes) {
  if (hi <= lo) return;
  const unsigned mis = (unsigned)(((16u - ((unsigned)(unsigned long long)(dst + lo) & 15u)) & 15u) >> 2);
  const long long head = lo + mis < hi ? lo + mis : hi;
  if (lo + lane < head) dst[lo + lane] = 0u;
  const long long nv = (hi - head) >> 2; /* 16-byte units */
  const long long tail = head + 4 * nv;
  if (tail + lane < hi) dst[tail + lane] = 0u;
  if (lane == 0 && nv > 0) {
    unsigned long long g = (unsigned long long)(dst + head);
    long long bytes = nv * 16;
    while (bytes > 0) {
      const uint32_t b = bytes < (long long)zbytes ? (uint32_t)bytes : zbytes;
      asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;"
                   ::"l"(g), "r"(zsm), "r"(b) : "memory");
      g += b;
      bytes -= b;
    }
    asm volatile("cp.async.bulk.commit_group;" ::: "memory");
  }
}

/* Wait until this thread's bulk copies are complete. */
__device__ __forceinline__ void bulk_wait() {
  asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
}

/* Split form with merged outputs, classify: zero the words of outputs 0..n-1 that tiles
 * g0 .. g1-1 of input `in` write, with bulk copies of zeros (bulk_zero_span). */
__device__ __forceinline__ void zero_chunk_bulk(const BgParams &p, int in, long long g0, long long g1,
                                                int n, int lane, uint32_t zsm, uint32_t zbytes) {
  if (!p.out) return;
  const long long first = p.tile_prefix[in];
  const long long W = (p.in_len[in] + 31) >> 5;
  long long lo = (g0 - first) * SW, hi = (g1 - first) * SW;
  if (hi > W) hi = W;
  uint32_t *dst = p.out + p.out_off[in];
  for (int o = 0; o < n; ++o, dst += p.out_stride) bulk_zero_span(dst, lo, hi, lane, zsm, zbytes);
}

/* Split form with merged outputs, classify: zero the words of outputs 0..n-1 that tiles
 * g0 .. g1-1 of input `in` write (what zero_outputs does tile by tile). */
__device__ __forceinline__ void zero_chunk(const BgParams &p, int in, long long g0, long long g1,
                                           int n, int lane) {
  if (!p.out) return;
  const long long first = p.tile_prefix[in];
  const long long W = (p.in_len[in] + 31) >> 5;
  long long lo = (g0 - first) * SW, hi = (g1 - first) * SW;
  if (hi > W) hi = W;
  uint32_t *dst = p.out + p.out_off[in];
  for (int o = 0; o < n; ++o, dst += p.out_stride) zero_span(dst, lo, hi, lane);
}

/* Split form, classify: store the run masks of a chunk's tiles (row `row`, positions
 * l0 .. l0 + ct - 1, kept by lane 0 in the warp's shared words rs[w * 32 + l]) with one
 * coalesced store per mask word, and the row summary (OR over its tiles) that the work-list
 * kernel reads: stored for a whole-row chunk, ORed into words the launch zeroed otherwise. */
__device__ __forceinline__ void flush_runs(const BgParams &p, long long row, int l0, int ct,
                                           const uint32_t *rs, uint32_t *rowrun, int lane) {
  __syncwarp();
  const long long rows = (p.n_tiles + 31) >> 5;
  const long long g = row * 32 + lane;
  const bool mine = lane >= l0 && lane < l0 + ct && g < p.n_tiles;
#pragma unroll
  for (int w = 0; w < BG_NRUN; ++w) {
    const uint32_t v = mine ? rs[w * 32 + lane] : 0u;
    if (mine) p.runs[(long long)w * p.n_tiles + g] = v;
    const uint32_t s = __reduce_or_sync(FULL, v);
    if (lane == 0) {
      if (ct >= 32) rowrun[(long long)w * rows + row] = s;
      else if (s) atomicOr(rowrun + (long long)w * rows + row, s);
    }
  }
  __syncwarp();
}

/* Split form: a part's accumulators hold only its own outputs (local index). */
__device__ __forceinline__ void acc_clear_n(uint32_t *acc, const Tile &t, int n) {
  for (int i = 0; i < n * WPT; ++i) acc[i * 32 + t.lane] = 0u;
}
__device__ __forceinline__ S acc_get(const uint32_t *acc, const Tile &t, int o) {
  S v;
#pragma unroll
  for (int j = 0; j < WPT; ++j) v.w[j] = acc[(o * WPT + j) * 32 + t.lane];
  return v;
}

__device__ __forceinline__ void acc_store(const BgParams &p, const Tile &t, const uint32_t *acc) {
  for (int o = 0; o < BG_NOUT; ++o) {
    S v;
#pragma unroll
    for (int j = 0; j < WPT; ++j) v.w[j] = acc[(o * WPT + j) * 32 + t.lane];
    store(p, t, o, v);
  }
}
#endif

}  // namespace bg
