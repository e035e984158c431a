/* CPU oracle and CPU baseline: word-parallel Pablo evaluator in plain C (test infrastructure).
 *
 * Executes the flat instruction list of include/bitgen_gb300.h (bg_instr) over one input on the
 * host, with the semantics of the reference's stream operators:
 *   bitwise ops            bitgen/template/template.py:27-61
 *   Advance                template.py:63-70 (zeros enter at position 0); Lookahead is its
 *                          mirror image (zeros enter past the end of the input)
 *   MatchStar              (((M & C) + C) ^ C) | M        template_torch.py:392-407
 *   ScanThru               (M + C) & ~C                   template_torch.py:377-389
 *   SEL                    (c & a) | (~c & b)             bitgen/inst/inst_sel.py:42-57
 *   while / if             any bit of the condition in the whole stream
 *                          bitgen/inst/inst_block_while.py:137-153, inst_block_if.py:314-342
 * Streams are little-endian bit vectors of 64-bit words (position p = bit p % 64 of word p / 64);
 * additions carry from word to word.  A program without while/if is evaluated block by block
 * (Advance tails and addition carries kept between blocks, the way icgrep runs Parabix code);
 * other programs are evaluated one instruction at a time over the whole stream.
 *
 * Output is written in the reference layout (uint32 words, position 32w + j at bit 31 - j).
 * One call is single-threaded; callers run groups / inputs on separate threads.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct bgc_instr {
  int32_t op, dst, a, b, c, shift;
} bgc_instr;

enum { OP_AND = 0, OP_OR, OP_XOR, OP_NOT, OP_SEL, OP_ADV, OP_MATCHSTAR, OP_SCANTHRU, OP_COPY,
       OP_WHILE, OP_IF, OP_LOOK };

#define BGC_OK 0
#define BGC_ERR_INVALID 1
#define BGC_ERR_NOMEM 6
#define BGC_ERR_ITER 4

static uint64_t transpose8(uint64_t x) {
  /* 8x8 bit-matrix transpose, row k = byte k, column c = bit c (Hacker's Delight 7-3) */
  uint64_t t;
  t = (x ^ (x >> 7)) & 0x00AA00AA00AA00AAull;
  x = x ^ t ^ (t << 7);
  t = (x ^ (x >> 14)) & 0x0000CCCC0000CCCCull;
  x = x ^ t ^ (t << 14);
  t = (x ^ (x >> 28)) & 0x00000000F0F0F0F0ull;
  x = x ^ t ^ (t << 28);
  return x;
}

/* basis planes (position order) of words [w0, w0 + nw) of the input */
static void basis_block(const uint8_t *data, int64_t n, int64_t w0, int64_t nw, uint64_t *planes[8]) {
  for (int64_t w = 0; w < nw; ++w) {
    uint64_t pw[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    const int64_t base = (w0 + w) * 64;
    for (int r = 0; r < 8; ++r) {
      const int64_t p = base + 8 * r;
      uint64_t x = 0;
      if (p + 8 <= n) {
        memcpy(&x, data + p, 8); /* little-endian hosts: byte k at bits 8k.. */
#if defined(__BYTE_ORDER__) && __BYTE_ORDER__ == __ORDER_BIG_ENDIAN__
        x = __builtin_bswap64(x);
#endif
      } else {
        for (int k = 0; k < 8 && p + k < n; ++k) x |= (uint64_t)data[p + k] << (8 * k);
      }
      const uint64_t y = transpose8(x); /* byte c, bit k = bit c of byte k */
      for (int b = 0; b < 8; ++b) pw[b] |= ((y >> (8 * (7 - b))) & 0xFFu) << (8 * r);
    }
    for (int b = 0; b < 8; ++b) planes[b][w] = pw[b];
  }
}

static uint32_t brev32(uint32_t x) {
  x = ((x >> 1) & 0x55555555u) | ((x & 0x55555555u) << 1);
  x = ((x >> 2) & 0x33333333u) | ((x & 0x33333333u) << 2);
  x = ((x >> 4) & 0x0F0F0F0Fu) | ((x & 0x0F0F0F0Fu) << 4);
  x = ((x >> 8) & 0x00FF00FFu) | ((x & 0x00FF00FFu) << 8);
  return (x >> 16) | (x << 16);
}

static int popc64(uint64_t x) { return __builtin_popcountll(x); }

typedef struct {
  const bgc_instr *code;
  int n_code;
  uint64_t **slot; /* slot pointers (each nw words)  */
  int64_t nw;      /* words per slot in this pass    */
  int64_t n;       /* characters in the input        */
  uint64_t **tail; /* per instruction: previous-block words of the Advance operand (block mode) */
  uint8_t *carry;  /* per instruction: addition carry (block mode)                              */
  int64_t max_iter;
  int status;
} Ctx;

static int any_bits(const Ctx *C, const uint64_t *x) {
  const int64_t full = C->n / 64, rem = C->n % 64;
  for (int64_t w = 0; w < full && w < C->nw; ++w)
    if (x[w]) return 1;
  if (rem && full < C->nw && (x[full] & ((1ull << rem) - 1))) return 1;
  return 0;
}

static void exec_range(Ctx *C, int pc, int end) {
  while (pc < end && C->status == BGC_OK) {
    const bgc_instr *I = &C->code[pc];
    uint64_t *d = I->dst >= 0 ? C->slot[I->dst] : NULL;
    const uint64_t *a = I->a >= 0 ? C->slot[I->a] : NULL;
    const uint64_t *b = I->b >= 0 ? C->slot[I->b] : NULL;
    const uint64_t *c = I->c >= 0 ? C->slot[I->c] : NULL;
    const int64_t nw = C->nw;
    switch (I->op) {
      case OP_AND: for (int64_t w = 0; w < nw; ++w) d[w] = a[w] & b[w]; break;
      case OP_OR: for (int64_t w = 0; w < nw; ++w) d[w] = a[w] | b[w]; break;
      case OP_XOR: for (int64_t w = 0; w < nw; ++w) d[w] = a[w] ^ b[w]; break;
      case OP_NOT: for (int64_t w = 0; w < nw; ++w) d[w] = ~a[w]; break;
      case OP_SEL: for (int64_t w = 0; w < nw; ++w) d[w] = (a[w] & b[w]) | (~a[w] & c[w]); break;
      case OP_COPY: if (d != a) memmove(d, a, (size_t)nw * 8); break;
      case OP_ADV: {
        const int64_t q = I->shift / 64;
        const int r = (int)(I->shift % 64);
        const int64_t k = q + 1;
        uint64_t *tl = C->tail ? C->tail[pc] : NULL; /* k previous words, oldest first */
        uint64_t keep[64];
        uint64_t *nt = NULL;
        if (tl) { /* the operand's last k words, saved before d (which may alias a) changes */
          nt = k <= 64 ? keep : (uint64_t *)malloc((size_t)k * 8);
          if (!nt) { C->status = BGC_ERR_NOMEM; return; }
          if (nw >= k) {
            memcpy(nt, a + nw - k, (size_t)k * 8);
          } else {
            memcpy(nt, tl + nw, (size_t)(k - nw) * 8);
            memcpy(nt + k - nw, a, (size_t)nw * 8);
          }
        }
        for (int64_t w = nw - 1; w >= 0; --w) {
          const int64_t i0 = w - q, i1 = w - q - 1;
          uint64_t cur, prev;
          if (i0 >= 0) cur = a[i0]; else cur = tl ? tl[k + i0] : 0;
          if (i1 >= 0) prev = a[i1]; else prev = tl ? tl[k + i1] : 0;
          d[w] = r ? ((cur << r) | (prev >> (64 - r))) : cur;
        }
        if (tl) {
          memcpy(tl, nt, (size_t)k * 8);
          if (nt != keep) free(nt);
        }
        break;
      }
      case OP_MATCHSTAR:
      case OP_SCANTHRU: {
        uint64_t cy = C->carry ? C->carry[pc] : 0;
        for (int64_t w = 0; w < nw; ++w) {
          const uint64_t m = a[w], cc = b[w];
          const uint64_t x = I->op == OP_MATCHSTAR ? (m & cc) : m;
          const uint64_t s1 = x + cc;
          const uint64_t c1 = s1 < x;
          const uint64_t s = s1 + cy;
          const uint64_t c2 = s < s1;
          cy = c1 | c2;
          d[w] = I->op == OP_MATCHSTAR ? ((s ^ cc) | m) : (s & ~cc);
        }
        if (C->carry) C->carry[pc] = (uint8_t)cy;
        break;
      }
      case OP_LOOK: { /* position p takes a[p + shift]; positions at or beyond n read as 0 */
        const int64_t q = I->shift / 64;
        const int r = (int)(I->shift % 64);
        const int64_t full = C->n / 64, rem = C->n % 64;
        for (int64_t w = 0; w < nw; ++w) {
          uint64_t v[2];
          for (int k = 0; k < 2; ++k) {
            const int64_t i = w + q + k;
            uint64_t x = i < nw ? a[i] : 0;
            if (i > full || (i == full && rem == 0)) x = 0;
            else if (i == full) x &= (1ull << rem) - 1;
            v[k] = x;
          }
          d[w] = r ? ((v[0] >> r) | (v[1] << (64 - r))) : v[0];
        }
        break;
      }
      case OP_WHILE: {
        int64_t it = 0;
        while (C->status == BGC_OK && any_bits(C, C->slot[I->a])) {
          if (C->max_iter > 0 && ++it > C->max_iter) {
            C->status = BGC_ERR_ITER;
            return;
          }
          exec_range(C, pc + 1, pc + 1 + I->shift);
        }
        pc += I->shift;
        break;
      }
      case OP_IF: {
        if (any_bits(C, C->slot[I->a]))
          exec_range(C, pc + 1, pc + 1 + I->shift);
        else
          exec_range(C, pc + 1 + I->shift, pc + 1 + I->shift + I->b);
        pc += I->shift + I->b;
        break;
      }
      default:
        C->status = BGC_ERR_INVALID;
        return;
    }
    ++pc;
  }
}

/* store words [w0, w0+nw) (64-bit, position order) of a result into the reference layout */
static void store_block(const uint64_t *x, int64_t w0, int64_t nw, int64_t n, uint32_t *out,
                        uint64_t *count) {
  const int64_t W32 = (n + 31) / 32;
  for (int64_t w = 0; w < nw; ++w) {
    uint64_t v = x[w];
    const int64_t p0 = (w0 + w) * 64;
    if (p0 >= n) break;
    if (n - p0 < 64) v &= (1ull << (n - p0)) - 1;
    if (count) *count += (uint64_t)popc64(v);
    if (out) {
      const int64_t o = 2 * (w0 + w);
      if (o < W32) out[o] = brev32((uint32_t)v);
      if (o + 1 < W32) out[o + 1] = brev32((uint32_t)(v >> 32));
    }
  }
}

/* Run `code` over data[0:n].  out: [n_out][ceil(n/32)] uint32 (may be NULL);
 * counts: [n_out] (may be NULL).  block_words: words per block for straight-line programs. */
int bgc_run(const bgc_instr *code, int n_code, int n_slots, const int *outs, int n_out,
            const uint8_t *data, int64_t n, uint32_t *out, uint64_t *counts, int64_t max_iter,
            int64_t block_words) {
  if (!code || n_slots < 10 || n < 0 || (n_out && !outs)) return BGC_ERR_INVALID;
  int control = 0;
  int64_t max_q = 0;
  for (int i = 0; i < n_code; ++i) {
    if (code[i].op == OP_WHILE || code[i].op == OP_IF || code[i].op == OP_LOOK) control = 1;
    if (code[i].op == OP_ADV && code[i].shift / 64 + 1 > max_q) max_q = code[i].shift / 64 + 1;
  }
  const int64_t NW = (n + 63) / 64;
  int64_t B = control ? (NW > 0 ? NW : 1) : (block_words > 0 ? block_words : 256);
  if (B > NW && NW > 0) B = NW;
  if (B < 1) B = 1;
  const int64_t W32 = (n + 31) / 32;
  if (counts) memset(counts, 0, sizeof(uint64_t) * (size_t)n_out);
  if (out) memset(out, 0, sizeof(uint32_t) * (size_t)n_out * (size_t)W32);
  uint64_t *pool = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)n_slots * (size_t)B);
  uint64_t **slot = (uint64_t **)malloc(sizeof(uint64_t *) * (size_t)n_slots);
  uint64_t **tail = NULL;
  uint8_t *carry = NULL;
  if (!pool || !slot) {
    free(pool);
    free(slot);
    return BGC_ERR_NOMEM;
  }
  for (int s = 0; s < n_slots; ++s) slot[s] = pool + (size_t)s * (size_t)B;
  if (!control) {
    tail = (uint64_t **)calloc((size_t)(n_code > 0 ? n_code : 1), sizeof(uint64_t *));
    carry = (uint8_t *)calloc((size_t)(n_code > 0 ? n_code : 1), 1);
    for (int i = 0; i < n_code; ++i)
      if (code[i].op == OP_ADV) tail[i] = (uint64_t *)calloc((size_t)(code[i].shift / 64 + 1), 8);
  }
  Ctx C;
  C.code = code;
  C.n_code = n_code;
  C.slot = slot;
  C.n = n;
  C.tail = tail;
  C.carry = carry;
  C.max_iter = max_iter;
  C.status = BGC_OK;
  for (int64_t w0 = 0; w0 < (NW > 0 ? NW : 1) && C.status == BGC_OK; w0 += B) {
    const int64_t nw = (NW - w0) < B ? (NW - w0) : B;
    if (nw <= 0) break;
    C.nw = nw;
    /* positions of this block relative to its start: the whole-stream tests use C.n, which is
       only meaningful when the block is the whole stream (programs with while/if) */
    uint64_t *planes[8];
    for (int k = 0; k < 8; ++k) planes[k] = slot[k];
    basis_block(data, n, w0, nw, planes);
    memset(slot[8], 0, (size_t)nw * 8);
    memset(slot[9], 0xFF, (size_t)nw * 8);
    exec_range(&C, 0, n_code);
    for (int o = 0; o < n_out; ++o)
      store_block(slot[outs[o]], w0, nw, n, out ? out + (size_t)o * (size_t)W32 : NULL,
                  counts ? counts + o : NULL);
  }
  if (tail) {
    for (int i = 0; i < n_code; ++i) free(tail[i]);
    free(tail);
  }
  free(carry);
  free(pool);
  free(slot);
  return C.status;
}
