/* bitgen_gb300: C ABI of the GB300 (sm_103a) bitstream execution engine.
 *
 * The entry points replace, one for one, what BitGen's CUDA backend binds for its hot path:
 *
 *   bg_transpose         <- byte_stream_transpose(bytestream, bitstream)
 *                           bitgen/template/cuda/pybind.cpp:9, bitgen/template/cuda/kernel.cu:102-124
 *   bg_program_create    <- CUDA_Kernel.init / init_single (NVRTC compile + module load)
 *                           bitgen/backend/cuda/cuda_kernel.py:64-171
 *   bg_program_destroy   <- CUDA_Kernel.free   bitgen/backend/cuda/cuda_kernel.py:400-406
 *   bg_plan_create       <- init_args (result / scratch allocation, kernel argument packing)
 *                           bitgen/backend/cuda/template/template.py:9-112
 *   bg_plan_launch       <- run_kernel / CUDA_Kernel.run (cuLaunchKernel)
 *                           template.py:116-121, cuda_kernel.py:411-427
 *   bg_plan_sync         <- the cuStreamSynchronize + checkCudaErrors after each run
 *                           cuda_kernel.py:35-47,411-427
 *   bg_plan_stats        <- the optional dyn_stats buffer of the generated kernel
 *                           bitgen/backend/cuda/template/template_dyn_stat.py:39-87
 *   bg_interp_*          <- the reference's whole-stream semantics of Pablo while/if
 *                           (bitgen/inst/inst_block_while.py:137-153, inst_block_if.py:314-342)
 *   bg_scan_noalloc      <- no counterpart in the reference (an allocation-free scan, below)
 *
 * All pointers to device memory are plain CUDA device pointers; `stream` is a cudaStream_t
 * (NULL = legacy default stream).  Every function returns a bg_status; none exits the process
 * (the reference's transpose calls exit() on a CUDA error, kernel.cu:7-15).
 * A bg_program / bg_plan must be used from one host thread at a time.
 */
#ifndef BITGEN_GB300_H
#define BITGEN_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum bg_status {
  BG_OK = 0,
  BG_ERR_INVALID = 1,  /* bad argument, shape or layout                           */
  BG_ERR_CUDA = 2,     /* a CUDA runtime call failed                              */
  BG_ERR_COMPILE = 3,  /* NVRTC rejected the program (see bg_program_log)         */
  BG_ERR_TIMEOUT = 4,  /* a bounded device wait (carry look-back) gave up         */
  BG_ERR_ALIGN = 5,    /* an input pointer or offset is not 16-byte aligned        */
  BG_ERR_NOMEM = 6,    /* device or host allocation failed                        */
  BG_ERR_DEVICE = 7,   /* kernel reported an internal inconsistency               */
  BG_ERR_CAPACITY = 8  /* a caller-provided output buffer was too small           */
} bg_status;

#define BG_INPUT_BYTES 0 /* raw bytes, transposed inside the scan kernel             */
#define BG_INPUT_BASIS 1 /* reference basis planes uint32 [8][W] per input            */

const char *bg_status_string(int status);
/* Human-readable detail of the last failing call on this host thread. */
const char *bg_last_error(void);
/* 1 if a CUDA device is usable by this process, 0 otherwise. */
int bg_device_available(void);

/* Byte -> basis transpose.  bytes: uint8 [n_inputs][n_bytes_padded] (n_bytes_padded % 32 == 0,
 * 16-byte aligned); basis: uint32 [n_inputs][8][n_bytes_padded / 32].  Plane i holds bit 7-i
 * of every byte; character 32w+j is bit 31-j of word w.  Asynchronous on `stream`. */
int bg_transpose(const uint8_t *bytes, uint32_t *basis, int64_t n_bytes_padded, int64_t n_inputs,
                 void *stream);

/* ---------------------------------------------------------------------------------------
 * Fused scan programs (CUDA C++ generated by bitgen_gb300.compiler, compiled with NVRTC for
 * sm_103a).  `source` may #include "bg_device.cuh" and "bg_params.h": the library supplies them.
 * ------------------------------------------------------------------------------------- */
typedef struct bg_program bg_program;
typedef struct bg_kernel_desc {
  const char *source;
  size_t source_len;
  const char *name;   /* __global__ entry point                                       */
  int32_t n_outputs;  /* output streams written by one launch                          */
  int32_t n_adds;     /* MatchStar / ScanThru additions (look-back record sets)         */
  int32_t halo_lanes; /* tile geometry: 32 lanes, the first halo_lanes and the last
                         tail_lanes re-computed; (32-halo-tail)*wpt words written       */
  int32_t wpt;        /* 32-bit words per lane                                          */
  int32_t block;      /* threads per CTA                                                */
  int32_t tail_lanes;
  int32_t n_pre;      /* additions 0..n_pre-1 get their carries from a pre-pass: the source
                         then also defines the kernel "<name>_pre" (0 = no pre-pass)      */
  int32_t n_run;      /* split form (> 0): the source defines "<name>_cls", which writes
                         n_run run-mask words per tile (and the pre-pass aggregates), and
                         "<name>" runs the parts on the tiles their masks select           */
  int32_t flags;      /* BG_PROGRAM_MERGES: parts OR into shared outputs, so every launch
                         needs out_streams (counts are taken from the bits a part adds)   */
  int32_t n_parts;    /* split form: part functions (work items are (part, 32 tiles))      */
} bg_kernel_desc;

#define BG_PROGRAM_MERGES 1

int bg_program_create(const bg_kernel_desc *desc, bg_program **out);
/* Compile only (no device needed): returns BG_OK or BG_ERR_COMPILE, log copied into log_buf. */
int bg_nvrtc_check(const char *source, size_t source_len, const char *name, char *log_buf,
                   size_t log_len);
/* Copies the NVRTC log (NUL-terminated, truncated to len) into buf. */
int bg_program_log(const bg_program *prog, char *buf, size_t len);
/* Registers, local memory and shared memory per thread/CTA of the compiled kernel. */
int bg_program_info(const bg_program *prog, int32_t *regs, int32_t *local_bytes,
                    int32_t *max_blocks_per_sm);
int bg_program_destroy(bg_program *prog);

/* Where the inputs and outputs of one launch live.  All arrays are host arrays, copied. */
typedef struct bg_layout {
  int32_t input_kind;     /* BG_INPUT_BYTES or BG_INPUT_BASIS                              */
  int32_t n_inputs;
  const int64_t *in_off;  /* [n_inputs] byte offset (bytes; multiple of 16) or word offset of
                             plane 0 (basis)                                               */
  const int64_t *in_len;  /* [n_inputs] characters in each input                          */
  int64_t basis_stride;   /* words between the 8 planes of one input (basis kind)          */
  const int64_t *out_off; /* [n_inputs] word offset of each input inside an output stream  */
  int64_t out_stride;     /* words between consecutive output streams                      */
} bg_layout;

typedef struct bg_plan bg_plan;
/* Plan for one fixed layout (tables uploaded synchronously). */
int bg_plan_create(bg_program *prog, const bg_layout *layout, bg_plan **out);
/* Plan with room for up to max_inputs inputs / max_tiles tiles, for layouts that change between
 * launches (batched and served scans); no layout is set yet. */
int bg_plan_reserve(bg_program *prog, int32_t input_kind, int32_t max_inputs, int64_t max_tiles,
                    bg_plan **out);
/* Set the layout of later launches: tables are staged in pinned memory and uploaded on `stream`
 * (stream-ordered before the next bg_plan_launch on the same stream). */
int bg_plan_set_layout(bg_plan *plan, const bg_layout *layout, void *stream);
/* Number of tiles one launch processes. */
int64_t bg_plan_tiles(const bg_plan *plan);
/* Bound (clock64 cycles, 0 = default of about 1 s) for every look-back wait of later launches.
 * debug_wait_tile >= 0 makes that tile first wait on a record no kernel writes, so that the
 * bound and the BG_ERR_TIMEOUT report can be exercised without faulting or hanging the GPU. */
int bg_plan_set_wait_limit(bg_plan *plan, int64_t spin_limit_cycles, int64_t debug_wait_tile);
/* Sparse output for later launches: every set bit of every output stream is also appended to
 * `positions` as (output << 52) | (input << 32) | position (unordered; limits: < 4095 outputs,
 * < 2^20 inputs, positions < 2^32).  capacity 0 turns it off.  Entries beyond the capacity are
 * dropped and bg_plan_sync reports BG_ERR_CAPACITY (the counts stay exact).
 * Positions-only launches (bg_plan_launch with out_streams NULL) of a program whose parts share
 * outputs (BG_PROGRAM_MERGES) need this call first: they count each set bit once through a
 * set of the positions found so far, which this call allocates in the plan (twice `capacity`
 * slots, rounded up to a power of two) and the launch clears.  `positions` may then be NULL:
 * counts only.  Beyond twice the capacity of distinct positions, bg_plan_sync reports
 * BG_ERR_CAPACITY and the counts are incomplete.  Such launches write no output streams: the
 * device traffic is the input, the positions and the counts. */
int bg_plan_set_positions(bg_plan *plan, unsigned long long *positions, int64_t capacity);
/* Number of positions the last launch on `stream` produced (waits for the stream). */
int bg_plan_positions_written(bg_plan *plan, void *stream, int64_t *written);
/* Work counters of the last launch on `stream` (waits for the stream); replaces the optional
 * `dyn_stats` buffer of the reference's generated kernel (bitgen/backend/cuda/template/
 * template_dyn_stat.py:39-87, filled at bitgen/codegen/gen_cuda.py:152-170), whose per-tile loop
 * counters have no meaning in this engine.  For each of the n_parts parts of a split-form
 * program: tiles_run[k] = tiles the execute pass ran part k on, rows[k] = 32-tile rows of its
 * work list.  Reads the plan's run masks back to the host (4 * n_run bytes per tile): not for
 * timed loops.  BG_ERR_INVALID for a single-kernel program, where every tile runs every term. */
int bg_plan_stats(bg_plan *plan, void *stream, int32_t n_parts, int64_t *tiles_run, int64_t *rows);
/* Enqueue one scan on `stream`: input is the device base of the bytes / basis planes;
 * out_streams (may be NULL; see bg_plan_set_positions for programs with BG_PROGRAM_MERGES)
 * receives n_outputs streams in the reference bit layout, positions at or beyond an input's
 * length cleared; counts (may be NULL) receives uint64 popcounts [n_outputs][n_inputs] (zeroed
 * by the call).  Only asynchronous work is enqueued, so the call can be captured into a CUDA
 * graph. */
int bg_plan_launch(bg_plan *plan, const void *input, uint32_t *out_streams,
                   unsigned long long *counts, void *stream);
/* Wait for `stream`, then report (and clear) device-side errors of earlier launches. */
int bg_plan_sync(bg_plan *plan, void *stream);
int bg_plan_destroy(bg_plan *plan);

/* ---------------------------------------------------------------------------------------
 * Allocation-free scan of one byte input.  No counterpart in the reference: BitGen always
 * allocates its outputs and working buffers per call.
 *
 * For callers that must not allocate device memory while they scan.  Examples are a process
 * whose device memory is owned by a pooling allocator with a hard budget, where a stray
 * cudaMalloc fails or escapes the pool's accounting, and a latency-bound loop, where
 * cudaFree's implicit device-wide synchronisation would stall every other stream.  The call
 * enqueues the same fused kernel as bg_plan_launch.  Its look-back records, launch tables and
 * state live in one fixed device array of BG_NOALLOC_SCRATCH_BYTES inside this library, not
 * in buffers of a plan.  Nothing is allocated and nothing is freed: no cudaMalloc, no
 * cudaFree, no memory pool.
 *
 *   prog         a program from bg_program_create, created on the current device;
 *   input        device bytes, 16-byte aligned; exactly n_bytes are read (n_bytes >= 0);
 *   out_streams  NULL, or n_outputs rows of out_stride >= ceil(n_bytes / 32) words, written in
 *                the reference bit layout (positions at or beyond n_bytes cleared);
 *   counts       NULL, or n_outputs uint64 popcounts (zeroed by the call);
 *   status       device uint32 (required); once the stream reaches the end of this call it
 *                holds the scan's device status bits: 0 on success, 1 if a carry look-back
 *                wait ran out of time, 2 if a look-back walked past the first tile.
 *
 * Limit: for T tiles of (32 - halo_lanes - tail_lanes) * wpt words and R = ceil(T / 32), the
 * scratch must hold max(1, additions) * T + ceil(3 * n_pre * R / 2) + ceil(n_run * T / 2) +
 * ceil(w / 2) 64-bit words out of BG_NOALLOC_RECORDS, where w = n_parts * (R + 1) + 512 +
 * n_run * R for the split form (n_run > 0) and 0 otherwise.  Larger inputs are rejected with BG_ERR_CAPACITY before
 * anything is enqueued, and bg_last_error() gives the sizes and the largest input that fits.
 * The first call on each device looks up the array's device address once
 * (cudaGetSymbolAddress) with that device current; make that first call before any stream
 * capture begins.  The address is kept for the life of the process: a device reset
 * (cudaDeviceReset) after that first call is not supported.
 * Every call on a device shares the one array.  The call clears what must start at zero,
 * including its own look-back records, and bumps the records' epoch.  Two calls whose work overlaps on the GPU (on different
 * streams, or from different host threads) race on the array and give wrong results.
 * Serialise them, for example on one stream.
 * ------------------------------------------------------------------------------------- */
#define BG_NOALLOC_SCRATCH_BYTES (4u << 20)
#define BG_NOALLOC_RECORDS (BG_NOALLOC_SCRATCH_BYTES / 8u - 32u)
int bg_scan_noalloc(const bg_program *prog, const uint8_t *input, int64_t n_bytes,
                    uint32_t *out_streams, int64_t out_stride, unsigned long long *counts,
                    uint32_t *status, void *stream);

/* ---------------------------------------------------------------------------------------
 * Whole-stream executor for programs that keep while / if blocks (global any-bit semantics).
 * The program is a flat instruction list:
 *   op = 0 AND, 1 OR, 2 XOR, 3 NOT, 4 SEL, 5 ADVANCE, 6 MATCHSTAR, 7 SCANTHRU, 8 COPY,
 *        9 WHILE (a = condition slot, shift = body length), 10 IF (a = condition slot,
 *        shift = then length, b = else length; else body follows the then body),
 *        11 LOOKAHEAD (position p takes a[p + shift]; zeros past the end of the input)
 *   dst/a/b/c are variable slots; slot 0..7 = basis0..7, slot 8 = all zeros, 9 = all ones.
 * ------------------------------------------------------------------------------------- */
typedef struct bg_instr {
  int32_t op, dst, a, b, c, shift;
} bg_instr;
typedef struct bg_interp bg_interp;
int bg_interp_create(const bg_instr *code, int32_t n_code, int32_t n_slots,
                     const int32_t *out_slots, int32_t n_outputs, bg_interp **out);
/* Runs the program over each input of the layout (basis kind or bytes kind), synchronously.
 * max_iterations bounds every while loop (0 = no bound); exceeding it returns BG_ERR_TIMEOUT. */
int bg_interp_run(bg_interp *prog, const bg_layout *layout, const void *input,
                  uint32_t *out_streams, unsigned long long *counts, int64_t max_iterations,
                  void *stream);
int bg_interp_destroy(bg_interp *prog);

#ifdef __cplusplus
}
#endif
#endif
