/* lfg.h -- C ABI of the GB300 (sm_103a) execute path for lean-fftw problems.
 *
 * This library executes lean-fftw's fast-engine transforms on the GPU: 1-D and batched
 * complex DFTs (binary64 by default) with the reference's own Stockham passes, twiddle
 * tables and generated butterfly codelets, so a binary64 plan with the same radix sequence
 * returns bit-identical results.  Problems are described with lean-fftw's FFI encoding.
 *
 * Conventions (lean-fftw docs/CONTRACT.md): unnormalised transforms; forward = sign -1;
 * complex data interleaved (re, im) unless a split layout is given by the spec's offsets.
 * Every entry point returns an lfg_status; unsupported problems return LFG_ERR_UNSUPPORTED
 * and never compute a different transform (lean-fftw docs/CONTRACT.md:44-45).  No C++
 * exception crosses this interface (host allocation failures return LFG_ERR_NOMEM).  Data
 * pointers must be aligned to a complex element: 16 bytes for binary64, 8 for binary32
 * (LFG_ERR_INVALID otherwise, before anything runs).
 */
#ifndef LFG_H
#define LFG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  LFG_OK = 0,
  LFG_ERR_UNSUPPORTED = 1, /* outside the supported problem domain (no plan)          */
  LFG_ERR_INVALID = 2,     /* malformed arguments (null pointer, bad spec length ...)  */
  LFG_ERR_CUDA = 3,        /* a CUDA runtime call failed                              */
  LFG_ERR_NOMEM = 4,       /* host or device allocation failed                        */
  LFG_ERR_TIMEOUT = 5      /* a bounded device-side wait gave up (binary32 tile copies) */
} lfg_status;

typedef enum { LFG_F64 = 0, LFG_F32 = 1 } lfg_precision;

/* Planning flags. */
#define LFG_ESTIMATE 0u      /* radix sequence with the fewest floating-point operations     */
#define LFG_MEASURE 1u       /* time the leading candidates on the device, keep the fastest */
#define LFG_PER_SIZE 2u      /* ragged: one launch per distinct size (the comparison point)  */
#define LFG_PER_SIZE_CONCURRENT 64u /* ragged, with LFG_PER_SIZE: the per-size launches spread
                                       over independent branches (streams / graph branches),
                                       so different sizes run at the same time */
#define LFG_NO_GRAPH 4u      /* ragged: launch directly instead of replaying a CUDA graph    */
#define LFG_ADJOINT 8u       /* r2c/c2r: exact cotangent scaling of the adjoint (see below)  */
#define LFG_NO_COMPENSATION 16u /* binary32: plain twiddle products in every pass             */
/* Testing the recovery path only: the binary32 persistent kernel's tile waits give up at
 * once (its bulk copies still land and are waited for before the kernel exits).  A call on
 * such a plan computes nothing useful; lfg_device_status then returns LFG_ERR_TIMEOUT. */
#define LFG_TEST_WAIT_GIVE_UP 32u
/* Run the kernels with runtime pass descriptors even where a kernel compiled for the plan's
 * geometry exists (binary32 power-of-two complex plans, and the rows and columns of binary32
 * real plans): the same bits, for comparing the two. */
#define LFG_GENERIC_KERNELS 128u

typedef struct lfg_plan lfg_plan;

/* Plan a problem given in lean-fftw's FFI encoding (LeanFFTW/FFI.lean:13-21, decoded as in
 * FFI.lean:32-47): doubles holding small integers
 *   [kind, sign, rank, vrank, inRe, inIm, outRe, outIm,
 *    (n, is, os) x rank, (n, is, os) x vrank, r2rkind x rank]
 * kind 0 = complex DFT (any rank and vector rank), 1 = rdft2 (r2c when sign < 0, c2r
 * otherwise; rank 1-2, vector rank <= 1), 2 = r2r (any rank, one kind per dimension, see
 * lfg_plan_r2r); strides and offsets
 * are in real scalars of the plan's precision (doubles for LFG_F64, as in the reference;
 * floats for LFG_F32), relative to the pointers later given to lfg_execute.  Replaces
 * `lfftw_generic_plan` (LeanFFTW/FFI.lean:50-52) for the kinds and layouts this library
 * executes.  A vector dimension of size 0 gives an empty plan (Core/Problem.lean:251-256).
 * Returns LFG_ERR_UNSUPPORTED (and *out = NULL) for anything else. */
lfg_status lfg_plan_spec(const double *spec, size_t nspec, lfg_precision precision,
                         unsigned flags, lfg_plan **out);

/* 1-D complex transform of size n, unit stride, interleaved, `howmany` contiguous
 * transforms (distance n).  sign < 0: forward.  The fast-engine entry point: replaces
 * `lfa_plan_measure(N, fwd, in, out)` (LeanFFTW/Asm/Planner.lean:293-302), which plans one
 * transform of a 13-smooth n; this version also batches. */
lfg_status lfg_plan_1d(size_t n, int sign, size_t howmany, lfg_precision precision,
                       unsigned flags, lfg_plan **out);

/* As lfg_plan_1d with an explicit radix sequence radices[0..npass) whose product is n
 * (each radix 2..16): the passes of lean-fftw's `refTransform fwd n radices`
 * (LeanFFTW/Gen/Stockham.lean:298-301).  Used by the autotuner and by parity tests. */
lfg_status lfg_plan_1d_radices(size_t n, int sign, size_t howmany, lfg_precision precision,
                               const int *radices, int npass, lfg_plan **out);

/* Real-input forward (r2c) and real-output backward (c2r) transforms, even n (13-smooth),
 * `howmany` contiguous lines: real lines of n scalars (double or float by `precision`),
 * complex lines of n/2+1 interleaved values.  The rank-2 versions transform n0 x n1 images (r2c along the last axis, then a
 * complex DFT along the first; c2r the reverse), images contiguous.  Replaces the generic
 * engine's rdft2 path (`planProblemCore`, LeanFFTW/Core/Problem.lean:222-236, and
 * `LineOp.apply`, :142-150); c2r ignores the imaginary parts of the self-conjugate bins
 * (docs/CONTRACT.md:20-23). */
lfg_status lfg_plan_r2c(size_t n, size_t howmany, lfg_precision precision, unsigned flags,
                        lfg_plan **out);
lfg_status lfg_plan_c2r(size_t n, size_t howmany, lfg_precision precision, unsigned flags,
                        lfg_plan **out);
lfg_status lfg_plan_r2c_2d(size_t n0, size_t n1, size_t howmany, lfg_precision precision,
                           unsigned flags, lfg_plan **out);
lfg_status lfg_plan_c2r_2d(size_t n0, size_t n1, size_t howmany, lfg_precision precision,
                           unsigned flags, lfg_plan **out);

/* Real-to-real transforms of one of libbench2's eleven kinds (numbering as lean-fftw's FFI,
 * LeanFFTW/FFI.lean:29-31): 0 R2HC, 1 HC2R, 2 DHT, 3 REDFT00, 4 REDFT01, 5 REDFT10,
 * 6 REDFT11, 7 RODFT00, 8 RODFT01, 9 RODFT10, 10 RODFT11; `howmany` contiguous lines of n
 * real scalars.  Computed as lean-fftw's generic engine defines them: an exact symmetric
 * embedding into a complex DFT of size 1, 2, 4 or 8 times n (`R2RKind.embed/extract`,
 * LeanFFTW/Core/Problem.lean:64-112), which must be 13-smooth.  Multi-dimensional r2r
 * problems (one kind per dimension) go through lfg_plan_spec with kind 2. */
lfg_status lfg_plan_r2r(size_t n, int kind, size_t howmany, lfg_precision precision,
                        unsigned flags, lfg_plan **out);

/* With LFG_ADJOINT, lfg_plan_r2c doubles its output bins 1..n/2-1 (the gradient of c2r) and
 * lfg_plan_c2r halves its input bins 1..n/2-1 (the gradient of r2c), both exactly, inside
 * the kernels: the adjoint of each transform is the other one with this cotangent scaling. */

/* Multiply the outputs of a complex plan by `scale` in the kernel's store (1 = off, the
 * default; normalised or orthonormal conventions and their adjoints). */
lfg_status lfg_set_scale(lfg_plan *plan, double scale);

/* Execute on device pointers, enqueued on `stream` (a cudaStream_t; NULL = legacy default
 * stream).  in == out is allowed.  Replaces `lfa_call(rec, in, out)`
 * (LeanFFTW/Asm/Kernels.lean:1203-1204) and `lfftw_generic_exec` (LeanFFTW/FFI.lean:56-58)
 * for device-resident data. */
lfg_status lfg_execute(const lfg_plan *plan, const void *in, void *out, void *stream);

/* In-place execution of a complex plan that allocates nothing.  No counterpart in the
 * reference: lean-fftw has no device memory to manage.  lfg_execute allocates a plan's
 * scratch buffer with cudaMalloc the first time an in-place two-group plan (n above one
 * CTA's shared memory) runs; callers that cannot allocate device memory themselves (runtimes
 * that route all device memory through their own pool and forbid cudaMalloc, or steady-state
 * loops that cannot take its implicit device synchronisation) use this entry point instead.
 * The intermediate goes to a 16 MiB array in static device memory (held by every GPU that
 * loads the library until the process exits), so n * howmany * (16 or 8) bytes must not exceed
 * 16 MiB for two-group plans (LFG_ERR_UNSUPPORTED otherwise).  The array's device address is
 * looked up on the first call on each device, so make that first call before any stream
 * capture.  All calls share the one array: calls whose executions overlap on the GPU race on
 * it.  `data` is the device buffer given to the plan as both input and output.  Only plans
 * that run as one or two Stockham pass groups are taken (1-D, 13-smooth, one batch
 * dimension); plans of other algorithms (prime factors above 13, split or strided layouts)
 * keep buffers of their own and are refused with LFG_ERR_UNSUPPORTED before anything runs. */
lfg_status lfg_execute_inplace_static(const lfg_plan *plan, void *data, void *stream);

/* Execute on host pointers: copies the spanned input to the device, transforms, copies the
 * output back, and returns when the output is in `out`.  The host-memory analogue of
 * `lfa_call` (LeanFFTW/Asm/Kernels.lean:1203-1204) as called by the libbench2 backend
 * (bench/backends/bench-leanfftw.c:284-288). */
lfg_status lfg_execute_host(const lfg_plan *plan, const void *in, void *out);

/* Synchronises with the device and reports whether a kernel of this plan gave up a bounded
 * wait (LFG_ERR_TIMEOUT; the flag is then cleared).  The binary32 persistent kernel waits on
 * its bulk copies with an iteration limit instead of spinning forever. */
lfg_status lfg_device_status(const lfg_plan *plan);

/* Release a plan and its device memory. */
void lfg_destroy(lfg_plan *plan);

/* Introspection (the analogue of LF_PLAN_SHOW, LeanFFTW/Asm/Planner.lean:299-300):
 * the radix sequence (up to max_radices entries), number of passes and of kernel groups,
 * and bytes of input and output per execution. */
typedef struct {
  int64_t n;            /* transform size (last dimension)                  */
  int64_t howmany;      /* number of transforms                              */
  int sign;
  int precision;
  int npass;
  int ngroups;          /* kernel launches per execution                     */
  int radices[24];
  int64_t in_bytes;     /* spanned input bytes per execution                 */
  int64_t out_bytes;    /* spanned output bytes per execution                */
  double flops;         /* binary64 instructions of the codelets per execution */
  int cluster_ctas;     /* a lone transform on a thread-block cluster: its CTAs (0: none) */
  int direct_groups;    /* binary32 groups run by the register-staged two-pass kernel   */
  int small_kernel;     /* 1: run by the warp-tile kernel (one butterfly, n <= 16, or a
                         * binary32 two-pass plan of n <= 32)                            */
} lfg_plan_info;

lfg_status lfg_get_plan_info(const lfg_plan *plan, lfg_plan_info *info);

/* ---- Ragged batches: many transforms of different sizes in one persistent launch ----
 *
 * `count` 1-D complex transforms, transform i of size sizes[i] (13-smooth, 2..2^24), unit
 * stride, its data starting at complex element in_offsets[i] / out_offsets[i] of the
 * buffers given at execution (NULL offsets: packed back to back in the given order).
 * Out of place only; outputs must not overlap.  lean-fftw plans and runs one size at a
 * time (bench/backends/bench-leanfftw.c:270-291, LeanFFTW/Asm/Planner.lean:224-286); this
 * plans the whole batch once and executes it as one CUDA-graph-replayed persistent kernel.
 * Each output is bit-identical to lean-fftw's refTransform for its size and the radix
 * sequence the plan picked (lfg_get_ragged_radices). */
typedef struct lfg_ragged lfg_ragged;

/* Autotuning knobs (NULL = defaults): complex elements per CTA tile, largest size run as a
 * single shared-memory pass group, and per-size radix overrides (n_over entries; entry j is
 * size over_n[j] with over_radices[24*j .. 24*j + over_npass[j])). */
typedef struct {
  int64_t tile_target;
  int64_t single_max;
  int n_over;
  const int64_t *over_n;
  const int *over_npass;
  const int *over_radices;
  int block_shape;      /* persistent-kernel block shape 0..4 (threads x CTAs per SM)   */
} lfg_ragged_tuning;

lfg_status lfg_plan_ragged(const int64_t *sizes, size_t count, const int64_t *in_offsets,
                           const int64_t *out_offsets, int sign, lfg_precision precision,
                           unsigned flags, const lfg_ragged_tuning *tuning, lfg_ragged **out);
lfg_status lfg_execute_ragged(const lfg_ragged *plan, const void *in, void *out, void *stream);
/* Host buffers: copies the spanned input in, executes, copies the spanned output back. */
lfg_status lfg_execute_ragged_host(const lfg_ragged *plan, const void *in, void *out);
void lfg_destroy_ragged(lfg_ragged *plan);

typedef struct {
  int64_t count;        /* transforms                                    */
  int64_t classes;      /* distinct sizes                                */
  int64_t items;        /* work items of the persistent kernel           */
  int64_t grid;         /* CTAs of the persistent kernel                 */
  int64_t smem_bytes;   /* shared memory per CTA                         */
  int64_t launches;     /* kernel launches per execution                 */
  int64_t in_bytes, out_bytes;
  int64_t points;       /* sum of the sizes                              */
  double flops;         /* binary64 instructions of the codelets         */
  int64_t tile_target;  /* schedule in use (chosen by LFG_MEASURE, given by a tuning, or */
  int64_t single_max;   /* the defaults): tile, single-group limit, block shape          */
  int64_t block_shape;
} lfg_ragged_info;

lfg_status lfg_get_ragged_info(const lfg_ragged *plan, lfg_ragged_info *info);
/* Radix sequence used for size n (npass = 0 if n is not in the batch). */
lfg_status lfg_get_ragged_radices(const lfg_ragged *plan, int64_t n, int *radices, int *npass);

/* Tuning cache ("wisdom").  No counterpart in lean-fftw, whose measuring planner re-times
 * every plan (LeanFFTW/Asm/Planner.lean:209-286); the calls follow FFTW's
 * fftw_import_wisdom_from_filename / fftw_export_wisdom_to_filename / fftw_forget_wisdom.
 * Every schedule LFG_MEASURE picks is remembered for the process, keyed by the problem, and a
 * later LFG_MEASURE plan of the same problem reuses it without timing.  With the environment
 * variable LFG_WISDOM naming a file, the table is read from it on first use and each new
 * choice is appended.  Import merges a file's entries (LFG_ERR_INVALID if it cannot be read);
 * export writes all entries; lfg_wisdom_count reports how many are held. */
lfg_status lfg_wisdom_import(const char *path);
lfg_status lfg_wisdom_export(const char *path);
void lfg_wisdom_forget(void);
size_t lfg_wisdom_count(void);

/* The radix sequence and pass grouping a default 1-D plan of size n would use, computed on
 * the host only (no device is touched): the analogue of printing the chosen plan with
 * LF_PLAN_SHOW (LeanFFTW/Asm/Planner.lean:299-300) without building it.  radices: room for 24
 * ints; *npass = the sequence length; *first_group = the passes of the first pass group
 * (*npass for a single group).  Sizes with a prime factor above 13 (generic or Bluestein
 * paths) and sizes outside 2..2^24 return LFG_ERR_UNSUPPORTED. */
lfg_status lfg_plan_layout(size_t n, lfg_precision precision, int *radices, int *npass,
                           int *first_group);

/* Split a ragged batch over nshards devices (no counterpart in the reference, which runs one
 * transform at a time on one host): transform i goes to shard[i] in 0..nshards-1, balancing
 * each shard's codelet operations (the binary64 kernels are bound by them; sizes outside the
 * fast engine count 5 n log2 n), largest transforms first.  Host only, deterministic, so every
 * rank computes the same split from the same sizes.  cost (nshards doubles, may be NULL)
 * receives each shard's operations. */
lfg_status lfg_shard_ragged(const int64_t *sizes, size_t count, int nshards, int *shard,
                            double *cost);

/* Human-readable text of a status, and the last error message of this thread. */
const char *lfg_strerror(lfg_status s);
const char *lfg_last_error(void);

/* cos/sin(2*pi*m/n) for m < n as binary64, interleaved, from exact integer arithmetic:
 * lean-fftw's `Trig.cosSin2PiTable` (LeanFFTW/Core/Trig.lean:131-134). out: 2n doubles. */
lfg_status lfg_cos_sin_table(uint64_t n, double *out);

/* ---- lean-fftw's fast-engine entry points, for the libbench2 backend ------------------
 * The same arguments as lean-fftw's `lfa_plan_measure` and `lfa_call`, in plain C.
 *
 * lfg_lfa_plan_measure replaces `lfa_plan_measure(N, fwd, in, out)`
 * (LeanFFTW/Asm/Planner.lean:293-302): plans a binary64 1-D complex transform of size N
 * (forward when fwd != 0) for the caller's host arrays at addresses in and out (in == out:
 * in place), measuring candidate schedules on the device (LFG_MEASURE).  As with the
 * reference, the arrays' contents may be overwritten (this implementation leaves them as they
 * are).  Returns an opaque record, or NULL where the reference returns its empty plan: N
 * outside 2..2^24 or with a prime factor above 13 (message in lfg_last_error()).
 *
 * lfg_lfa_call has the signature and meaning of `lfa_call(record, in, out)`
 * (LeanFFTW/Asm/Kernels.lean:1203-1204, bench/backends/bench-leanfftw.c:284-288): the transform
 * of the host array in (2N doubles, interleaved) written to out, returning when out holds it.
 * It returns nothing, as lfa_call; lfg_lfa_status(record) gives the status of the record's last
 * call.  lfg_lfa_release frees the record (the reference's lean_dec of its plan array). */
const void *lfg_lfa_plan_measure(size_t N, uint8_t fwd, size_t in, size_t out);
void lfg_lfa_call(const void *record, const double *in, double *out);
lfg_status lfg_lfa_status(const void *record);
void lfg_lfa_release(const void *record);

#ifdef __cplusplus
}
#endif

#endif /* LFG_H */
