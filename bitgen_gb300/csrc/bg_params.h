/* Launch parameters shared by the host runtime and the generated sm_103a kernels.
 *
 * One launch scans many inputs (one for the reference's single-input path, thousands in the
 * batched form).  Every input is cut into tiles of (32 - HL) * WPT output words; a warp owns
 * one tile at a time and computes it over 32 lanes * WPT words, the first HL lanes being a
 * halo re-computed from the previous tile's words.  Carries of MatchStar/ScanThru additions
 * that cross a tile boundary are exchanged through per-addition look-back records.
 */
#ifndef BG_PARAMS_H
#define BG_PARAMS_H

#ifdef __CUDACC_RTC__
typedef unsigned char uint8_t;
typedef unsigned int uint32_t;
typedef int int32_t;
typedef long long int64_t;
typedef unsigned long long uint64_t;
#else
#include <stdint.h>
#endif

#define BG_INPUT_BYTES 0 /* raw bytes; the kernel transposes them itself            */
#define BG_INPUT_BASIS 1 /* 8 basis planes per input, reference layout [8][W] uint32 */

/* status bits written by kernels into state[1] */
#define BG_DEV_ERR_TIMEOUT 1u /* a look-back wait ran out of time                    */
#define BG_DEV_ERR_CHAIN 2u   /* a look-back walked past the first tile of its input */
#define BG_DEV_ERR_CAPACITY 4u /* the match-position buffer was too small             */
#define BG_DEV_ERR_SETFULL 8u  /* the position set ran out of slots (counts incomplete) */

typedef struct BgParams {
  const uint8_t *in_bytes;   /* BG_INPUT_BYTES: base of all inputs                        */
  const uint32_t *in_basis;  /* BG_INPUT_BASIS: base of all basis planes                  */
  const int64_t *in_off;     /* [n_inputs] byte offset (bytes) / word offset of plane 0   */
  const int64_t *in_len;     /* [n_inputs] characters in the input                         */
  const int64_t *tile_prefix;/* [n_inputs + 1] first global tile of each input            */
  const int64_t *out_off;    /* [n_inputs] word offset of the input inside each stream    */
  uint32_t *out;             /* output streams (reference bit layout) or NULL             */
  unsigned long long *counts;/* [n_outputs][n_inputs] popcounts, or NULL                  */
  unsigned long long *records;/* [n_adds][n_tiles] look-back records                      */
  uint32_t *state;           /* [0] tile counter, [1] status, [2..3] epoch (u64),
                                [4..5] a record no kernel ever writes (wait-limit test),
                                [6..7] match positions written (u64)                         */
  unsigned long long *positions; /* sparse output or NULL: (output << 52 | input << 32 | pos) */
  int64_t pos_capacity;
  unsigned long long *pos_set; /* launches without output streams of a program whose parts
                                  share outputs: open-addressed set of the positions set so far
                                  (all ones = empty slot, cleared by the classify pass), so that
                                  a bit two parts set is counted once; NULL otherwise          */
  int64_t pos_set_mask;      /* slots - 1 (slots a power of two)                           */
  int64_t basis_stride;      /* words between the basis planes of one input               */
  int64_t out_stride;        /* words between two output streams                          */
  int64_t n_tiles;
  int64_t spin_limit;        /* clock64 cycles a look-back wait may take before giving up */
  int64_t debug_wait_tile;   /* tile that first waits on the never-written record, or -1 */
  uint32_t *runs;            /* split form: [n_run][n_tiles] per-tile run masks, or NULL   */
  uint32_t *pre_bits;        /* pre-pass bitmaps, 3 * ceil(n_tiles / 32) words per addition */
  uint32_t *work;            /* split form, R = ceil(n_tiles / 32) rows of 32 tiles, H =
                                BG_WORK_HEAD: [0, H) the execute pass's claim counters (one
                                per group of SMs, BG_CLAIM_STRIDE words apart);
                                [H + p] = number of rows part p runs on; at
                                H + n_parts + p * R those rows (ascending); at
                                H + n_parts * (1 + R) the OR of each row's run masks, [n_run][R] */
  int32_t n_inputs;
  int32_t input_kind;
  int32_t chunk_tiles;       /* tiles per warp chunk in the classify / pre-pass kernels:
                                1..32, a power of two (the runtime's choice per launch)       */
} BgParams;

/* Words before the part counts in BgParams.work: the execute pass's claim counters, one per
 * group of SMs (at most 16), each in its own 128-byte line so that the groups' atomic claims
 * do not queue on one line. */
#define BG_CLAIM_STRIDE 32
#define BG_WORK_HEAD (16 * BG_CLAIM_STRIDE)

#endif
