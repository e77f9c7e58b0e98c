/* libbench2 backend for the GB300 execute path (liblfg.so): the same problem space and the
 * same two-engine split as lean-fftw's own backend (bench/backends/bench-leanfftw.c).
 *
 *  - 1-D complex transforms of unit stride, interleaved, in place or out of place, of a
 *    13-smooth size 2..2^24 run through the fast-engine entry points: lfg_lfa_plan_measure
 *    at setup, lfg_lfa_call in the timed loop (the reference's lfa_plan_measure / lfa_call,
 *    bench-leanfftw.c:225-297);
 *  - every other problem goes through lean-fftw's FFI problem encoding
 *    (LeanFFTW/FFI.lean:13-47): each side's spanned range of doubles (two ranges for split
 *    complex data) is staged back to back in a private host buffer, the real and imaginary
 *    bases become offsets into it, lfg_plan_spec plans the problem and lfg_execute_host runs
 *    it on the staging buffers; the output ranges are copied back.
 *
 * Built against libbench2's bench-user.h this links into libbench2's benchmark program;
 * the tests build it against a stand-in header (tests/libbench2_stub) and drive
 * can_do / setup / doit / done directly. */
#include "libbench2/bench-user.h"

#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "lfg.h"

BEGIN_BENCH_DOC
BENCH_DOC("name", "lean-fftw-gb300")
BENCH_DOC("version", "0.2")
BENCH_DOC("notes", "lean-fftw's execute path on a GB300: fast engine for 1-D complex "
                   "13-smooth sizes, FFI problem encoding for the rest")
END_BENCH_DOC

static const void *fast_rec = 0;   /* fast-engine record (lfg_lfa_plan_measure) */
static lfg_plan *spec_plan = 0;    /* everything else (lfg_plan_spec) */

/* One side of a problem: bases of the real and imaginary parts, and the number of doubles
 * per unit of the problem's strides (2 for interleaved complex data, 1 otherwise). */
typedef struct {
     double *re, *im;
     int real;
     int mul;
} side_t;

static int is_smooth13(size_t n)
{
     static const size_t primes[] = { 2, 3, 5, 7, 11, 13 };
     size_t i;
     for (i = 0; i < sizeof primes / sizeof primes[0]; ++i)
          while (n % primes[i] == 0) n /= primes[i];
     return n == 1;
}

static int fast_engine_problem(const bench_problem *p)
{
     if (p->kind != PROBLEM_COMPLEX || p->split) return 0;
     if (p->sz->rnk != 1 || p->vecsz->rnk != 0) return 0;
     if (p->sz->dims[0].is != 1 || p->sz->dims[0].os != 1) return 0;
     return p->sz->dims[0].n >= 2 && (size_t) p->sz->dims[0].n <= ((size_t) 1 << 24) &&
            is_smooth13((size_t) p->sz->dims[0].n);
}

static void make_sides(const bench_problem *p, side_t *si, side_t *so)
{
     double *ri = (double *) p->in, *ro = (double *) p->out;
     if (p->kind == PROBLEM_R2R) {
          si->re = si->im = ri; so->re = so->im = ro;
          si->real = so->real = 1;
          si->mul = so->mul = 1;
     } else if (p->kind == PROBLEM_COMPLEX) {
          si->real = so->real = 0;
          if (p->split) {
               si->re = ri; si->im = p->ini ? (double *) p->ini : ri + p->iphyssz;
               so->re = ro; so->im = p->outi ? (double *) p->outi : ro + p->ophyssz;
               si->mul = so->mul = 1;
          } else {
               si->re = ri; si->im = ri + 1;
               so->re = ro; so->im = ro + 1;
               si->mul = so->mul = 2;
          }
     } else {
          /* rdft2: the real side, and the half spectrum (n/2 + 1 along the last axis) on the
           * complex side, whose split imaginary part follows its real part */
          const int nl = p->sz->dims[p->sz->rnk - 1].n;
          const double total = tensor_sz(p->sz) * tensor_sz(p->vecsz);
          const long half = (long) (total / nl) * (nl / 2 + 1);
          side_t *rs = p->sign < 0 ? si : so, *cs = p->sign < 0 ? so : si;
          double *cb = p->sign < 0 ? ro : ri;
          rs->re = rs->im = p->sign < 0 ? ri : ro;
          rs->real = 1;
          rs->mul = 1;
          cs->real = 0;
          cs->re = cb;
          if (p->split) { cs->im = cb + half; cs->mul = 1; }
          else { cs->im = cb + 1; cs->mul = 2; }
     }
}

/* Offsets (in units of the problem's strides) of the lowest and highest element of one side. */
static void stride_span(const bench_problem *p, int output, int half_last, long *lo, long *hi)
{
     int d;
     *lo = *hi = 0;
     for (d = 0; d < p->sz->rnk + p->vecsz->rnk; ++d) {
          const bench_iodim *io = d < p->sz->rnk ? &p->sz->dims[d] : &p->vecsz->dims[d - p->sz->rnk];
          long n = io->n;
          const long s = output ? io->os : io->is;
          if (half_last && d == p->sz->rnk - 1) n = n / 2 + 1;
          if (n > 1) {
               if (s > 0) *hi += (n - 1) * s;
               else *lo += (n - 1) * s;
          }
     }
}

/* Where a side's data lives: one range of doubles (real data, or interleaved complex data,
 * whose imaginary parts sit inside it), or two ranges of equal length (split complex data;
 * the real and imaginary arrays may be separate allocations).  The library runs on a private
 * staging buffer holding the range(s) back to back, so nothing outside the caller's own
 * elements is ever read or written. */
typedef struct {
     double *part[2];   /* start of each range in the caller's memory */
     size_t len;        /* doubles per range */
     int nparts;
     double off_re, off_im;   /* FFI offsets of the re / im bases in the staging buffer */
     double *stage;
} staged_t;

static void stage_layout(const side_t *s, long lo, long hi, staged_t *st)
{
     st->len = (size_t) ((hi - lo) * s->mul + (s->real || s->mul == 1 ? 1 : 2));
     st->part[0] = s->re + lo * s->mul;
     st->nparts = (!s->real && s->mul == 1) ? 2 : 1;
     st->part[1] = st->nparts == 2 ? s->im + lo * s->mul : 0;
     st->off_re = (double) (-lo * s->mul);
     st->off_im = st->nparts == 2 ? (double) st->len - (double) (lo * s->mul)
                                  : st->off_re + (s->real ? 0 : 1);
     st->stage = 0;
}

static void stage_copy(staged_t *st, int to_stage)
{
     int k;
     for (k = 0; k < st->nparts; ++k) {
          if (to_stage) memcpy(st->stage + k * st->len, st->part[k], st->len * sizeof(double));
          else memcpy(st->part[k], st->stage + k * st->len, st->len * sizeof(double));
     }
}

static staged_t stin, stout;

/* lean-fftw's FFI encoding of the problem (LeanFFTW/FFI.lean:13-21), with the offsets of the
 * staging layouts; returns the number of doubles written. */
static int encode(const bench_problem *p, double *spec, staged_t *si_st, staged_t *so_st)
{
     side_t si, so;
     long ilo, ihi, olo, ohi;
     int k = 0, d;
     const int r = p->sz->rnk, v = p->vecsz->rnk;
     make_sides(p, &si, &so);
     stride_span(p, 0, p->kind == PROBLEM_REAL && p->sign > 0, &ilo, &ihi);
     stride_span(p, 1, p->kind == PROBLEM_REAL && p->sign < 0, &olo, &ohi);
     stage_layout(&si, ilo, ihi, si_st);
     stage_layout(&so, olo, ohi, so_st);
     spec[k++] = p->kind == PROBLEM_COMPLEX ? 0 : p->kind == PROBLEM_REAL ? 1 : 2;
     spec[k++] = p->sign;
     spec[k++] = r;
     spec[k++] = v;
     spec[k++] = si_st->off_re;
     spec[k++] = si_st->off_im;
     spec[k++] = so_st->off_re;
     spec[k++] = so_st->off_im;
     for (d = 0; d < r + v; ++d) {
          const bench_iodim *io = d < r ? &p->sz->dims[d] : &p->vecsz->dims[d - r];
          spec[k++] = io->n;
          spec[k++] = (double) io->is * si.mul;
          spec[k++] = (double) io->os * so.mul;
     }
     for (d = 0; d < r; ++d) spec[k++] = p->kind == PROBLEM_R2R ? (double) p->k[d] : 0.0;
     return k;
}

static lfg_plan *plan_problem(const bench_problem *p, staged_t *si_st, staged_t *so_st)
{
     double spec[8 + 4 * 64];
     lfg_plan *plan = 0;
     int nspec;
     if (p->sz->rnk + p->vecsz->rnk > 64) return 0;
     nspec = encode(p, spec, si_st, so_st);
     if (lfg_plan_spec(spec, (size_t) nspec, LFG_F64, LFG_ESTIMATE, &plan) != LFG_OK) return 0;
     return plan;
}

int can_do(bench_problem *p)
{
     staged_t a, b;
     lfg_plan *plan;
     if (!BENCH_FINITE_RNK(p->sz->rnk) || !BENCH_FINITE_RNK(p->vecsz->rnk)) return 0;
     if (fast_engine_problem(p)) return 1;
     plan = plan_problem(p, &a, &b);    /* what lfg_plan_spec accepts (nothing is touched) */
     if (!plan) return 0;
     lfg_destroy(plan);
     return 1;
}

void setup(bench_problem *p)
{
     if (fast_engine_problem(p)) {
          fast_rec = lfg_lfa_plan_measure((size_t) p->sz->dims[0].n, (uint8_t) (p->sign < 0),
                                          (size_t) p->in, (size_t) p->out);
          if (fast_rec) return;
     }
     spec_plan = plan_problem(p, &stin, &stout);
     if (spec_plan) {
          stin.stage = (double *) malloc(stin.nparts * stin.len * sizeof(double));
          stout.stage = (double *) malloc(stout.nparts * stout.len * sizeof(double));
     }
     if (!spec_plan || !stin.stage || !stout.stage) {
          fprintf(stderr, "lean-fftw-gb300: problem not supported: %s\n", lfg_last_error());
          bench_exit(1);
     }
}

void doit(int iter, bench_problem *p)
{
     int it;
     if (fast_rec) {
          const double *in = (const double *) p->in;
          double *out = (double *) p->out;
          for (it = 0; it < iter; ++it) lfg_lfa_call(fast_rec, in, out);
          if (lfg_lfa_status(fast_rec) != LFG_OK) {
               fprintf(stderr, "lean-fftw-gb300: %s\n", lfg_last_error());
               bench_exit(1);
          }
          return;
     }
     for (it = 0; it < iter; ++it) {
          /* the output ranges come along too: elements between a strided output's own keep
           * the caller's values */
          stage_copy(&stin, 1);
          stage_copy(&stout, 1);
          if (lfg_execute_host(spec_plan, stin.stage, stout.stage) != LFG_OK) {
               fprintf(stderr, "lean-fftw-gb300: %s\n", lfg_last_error());
               bench_exit(1);
               return;
          }
          stage_copy(&stout, 0);
     }
}

void done(bench_problem *p)
{
     (void) p;
     if (fast_rec) lfg_lfa_release(fast_rec);
     if (spec_plan) lfg_destroy(spec_plan);
     free(stin.stage);
     free(stout.stage);
     stin.stage = stout.stage = 0;
     fast_rec = 0;
     spec_plan = 0;
}

void main_init(int *argc, char ***argv)
{
     (void) argc;
     (void) argv;
}

void initial_cleanup(void) {}
void final_cleanup(void) {}
