/* ORACLE (test infrastructure only; never linked into the product).
 *
 * CPU restatements of lean-fftw's transforms, used to check the GPU kernels:
 *
 *  1. lfo_ref_transform: `refTransform` / `stockhamWith floatArith` / `passWith` /
 *     `bflyInputs` (LeanFFTW/Gen/Stockham.lean:263-301), the binary64 reference that
 *     lean-fftw's fast engine reproduces bit for bit.  The butterfly kernels of radix 2, 4,
 *     8 and 16 are lean-fftw's own generated kernels (codelets_native.c, written from
 *     LeanFFTW/Native/Kernels.lean); the other radices come from the restated codelet
 *     generator (codelets_gen.c).  Both are evaluated operand for operand with fma(); this
 *     file must be compiled with -ffp-contract=off.
 *  2. lfo_generic_dft: the generic engine, `exec floatOps (mkPlan floatOps fwd
 *     (primeFactors n))` (LeanFFTW/Core/Alg.lean:236-254, Core/FloatOps.lean:52-68,
 *     Core/Problem.lean:126-127), which lean-fftw runs for r2c/c2r and rank >= 2.
 *  3. lfo_dd_dft: an extended-precision (double-double) mixed-radix DFT, the accuracy
 *     oracle for relative L2 errors.  Error-free transformations after Knuth (TwoSum) and
 *     Dekker (TwoProduct, here through fma); accurate addition as in the QD library of
 *     Hida, Li and Bailey.
 *
 * All arrays are interleaved complex (re, im) doubles.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef void (*lfo_codelet_fn)(const double *x, double *y);
typedef void (*lfo_pass_fn)(long N, long ns, const double *tw, const double *z, double *o);
lfo_codelet_fn lfo_native_codelet(int fwd, int R, int tw);
lfo_pass_fn lfo_native_pass(int fwd, int R, int tw);
lfo_codelet_fn lfo_gen_codelet(int fwd, int R, int tw);
lfo_pass_fn lfo_gen_pass(int fwd, int R, int tw);

/* The butterfly of radix R: lean-fftw's generated kernel where it ships one, else the
 * restated generator's. */
lfo_codelet_fn lfo_codelet(int fwd, int R, int tw)
{
     lfo_codelet_fn f = lfo_native_codelet(fwd, R, tw);
     return f ? f : lfo_gen_codelet(fwd, R, tw);
}

static lfo_pass_fn lfo_pass(int fwd, int R, int tw)
{
     lfo_pass_fn f = lfo_native_pass(fwd, R, tw);
     return f ? f : lfo_gen_pass(fwd, R, tw);
}

/* Evaluate one butterfly (x: 2R data values, then 2(R-1) twiddle values when tw; y: 2R). */
int lfo_bfly(int fwd, int R, int tw, int native, const double *x, double *y)
{
     lfo_codelet_fn f = native ? lfo_native_codelet(fwd, R, tw) : lfo_gen_codelet(fwd, R, tw);
     if (!f) return -1;
     f(x, y);
     return 0;
}

/* ------------------------------------------------------------------ 1. refTransform */

/* One Stockham pass (Stockham.lean:276-284): butterfly j = b*ns + k reads z[j + r*N/R] and,
 * for t >= 1, the twiddles tw[2r*ns + k], tw[(2r+1)*ns + k] (r < R-1); its output r goes to
 * position b*ns*R + k + r*ns. */
static int ref_pass(int fwd, long N, int R, long ns, const double *tw, const double *z,
                    double *o)
{
     lfo_pass_fn pf = lfo_pass(fwd, R, tw != NULL);
     if (pf) {   /* the generated pass with the codelet inlined */
          pf(N, ns, tw, z, o);
          return 0;
     }
     lfo_codelet_fn f = lfo_codelet(fwd, R, tw != NULL);
     double x[4 * 64], y[2 * 64];
     long NR = N / R, j;
     int r;
     if (!f || R > 64) return -1;
     for (j = 0; j < NR; ++j) {
          long k = j % ns, b = j / ns;
          for (r = 0; r < R; ++r) {
               x[2 * r] = z[2 * (j + r * NR)];
               x[2 * r + 1] = z[2 * (j + r * NR) + 1];
          }
          if (tw)
               for (r = 0; r < R - 1; ++r) {
                    x[2 * R + 2 * r] = tw[2 * r * ns + k];
                    x[2 * R + 2 * r + 1] = tw[(2 * r + 1) * ns + k];
               }
          f(x, y);
          for (r = 0; r < R; ++r) {
               long c = b * ns * R + k + r * ns;
               o[2 * c] = y[2 * r];
               o[2 * c + 1] = y[2 * r + 1];
          }
     }
     return 0;
}

/* refTransform fwd N rs on `batch` contiguous transforms (batch stride 2N doubles).
 * tws[t] is the twiddle table of pass t (t >= 1; tws[0] unused), laid out as
 * passTwiddles (LeanFFTW/Core/FastPlan.lean:163-173).  work: 2N doubles per thread. */
int lfo_ref_transform(int fwd, long N, const int *rs, int npass, const double *const *tws,
                      const double *in, double *out, long batch, int nthreads)
{
     int err = 0;
     long bi;
     if (nthreads < 1) nthreads = 1;
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 1) reduction(| : err)
     for (bi = 0; bi < batch; ++bi) {
          double *w0 = (double *) malloc(sizeof(double) * 4 * (size_t) N);
          double *a = w0, *bb = w0 + 2 * N;
          long ns = 1;
          int t;
          if (!w0) { err |= 1; continue; }
          memcpy(a, in + 2 * N * bi, sizeof(double) * 2 * (size_t) N);
          for (t = 0; t < npass; ++t) {
               double *tmp;
               err |= ref_pass(fwd, N, rs[t], ns, t >= 1 ? tws[t] : NULL, a, bb) != 0;
               tmp = a; a = bb; bb = tmp;
               ns *= rs[t];
          }
          memcpy(out + 2 * N * bi, a, sizeof(double) * 2 * (size_t) N);
          free(w0);
     }
     return err ? -1 : 0;
}

/* refTransform over a ragged batch: transform i has class cls[i] (size cN[c], radices
 * crs[c][0..cnp[c]), pass tables ctw[c][t]) and lives at complex offsets ioff[i] / ooff[i].
 * One transform per thread. */
int lfo_ref_ragged(int fwd, long ncls, const long *cN, const int *cnp, const int *const *crs,
                   const double *const *const *ctw, long count, const long *cls,
                   const long *ioff, const long *ooff, const double *in, double *out,
                   int nthreads)
{
     int err = 0;
     long i;
     (void) ncls;
     if (nthreads < 1) nthreads = 1;
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 4) reduction(| : err)
     for (i = 0; i < count; ++i) {
          long c = cls[i], N = cN[c];
          double *w0 = (double *) malloc(sizeof(double) * 4 * (size_t) N);
          double *a = w0, *bb = w0 + 2 * N;
          long ns = 1;
          int t;
          if (!w0) { err |= 1; continue; }
          memcpy(a, in + 2 * ioff[i], sizeof(double) * 2 * (size_t) N);
          for (t = 0; t < cnp[c]; ++t) {
               double *tmp;
               err |= ref_pass(fwd, N, crs[c][t], ns, t >= 1 ? ctw[c][t] : NULL, a, bb) != 0;
               tmp = a; a = bb; bb = tmp;
               ns *= crs[c][t];
          }
          memcpy(out + 2 * ooff[i], a, sizeof(double) * 2 * (size_t) N);
          free(w0);
     }
     return err ? -1 : 0;
}

/* ------------------------------------------------------------------ 2. generic engine */

/* Textbook product with four rounded products (FloatOps.lean:52-53). */
static inline void fc_mul(double ar, double ai, double br, double bi, double *cr, double *ci)
{
     double p1 = ar * br, p2 = ai * bi, p3 = ar * bi, p4 = ai * br;
     *cr = p1 - p2;
     *ci = p3 + p4;
}

/* exec (Alg.lean:245-254) over the plan mkPlan fwd fs (Alg.lean:236-242).  x is read at
 * x[2*stride*j]; twiddles of level size n are cosSin2Pi(k, n), imaginary negated (never
 * to -0.0) when fwd (floatTw, FloatOps.lean:56-58); they come from the table of the full
 * size Ntab (tab[2*m] = cos, tab[2*m+1] = sin of 2*pi*m/Ntab), m = k*Ntab/n. */
static void gen_exec(int fwd, const int *fs, int nf, const double *x, long stride,
                     double *out, const double *tab, long Ntab)
{
     long n = 1, k, j;
     int i;
     for (i = 0; i < nf; ++i) n *= fs[i];
     if (nf <= 1) {
          /* direct leaf: out[k] = sum_j w[j*k mod n] * x[j], summed from zero */
          for (k = 0; k < n; ++k) {
               double accr = 0.0, acci = 0.0;
               for (j = 0; j < n; ++j) {
                    long m = (j * k % n) * (Ntab / n);
                    double wr = tab[2 * m], wi = tab[2 * m + 1], pr, pi;
                    if (fwd) wi = wi == 0.0 ? 0.0 : -wi;
                    fc_mul(wr, wi, x[2 * stride * j], x[2 * stride * j + 1], &pr, &pi);
                    accr = accr + pr;
                    acci = acci + pi;
               }
               out[2 * k] = accr;
               out[2 * k + 1] = acci;
          }
          return;
     }
     {
          int r = fs[0];
          long m = n / r, j1;
          double *ys = (double *) malloc(sizeof(double) * 2 * (size_t) n);
          for (j1 = 0; j1 < r; ++j1)
               gen_exec(fwd, fs + 1, nf - 1, x + 2 * stride * j1, stride * r, ys + 2 * m * j1,
                        tab, Ntab);
          for (k = 0; k < n; ++k) {
               double accr = 0.0, acci = 0.0;
               for (j1 = 0; j1 < r; ++j1) {
                    long mm = (j1 * k % n) * (Ntab / n);
                    double wr = tab[2 * mm], wi = tab[2 * mm + 1], pr, pi;
                    const double *y = ys + 2 * (m * j1 + k % m);
                    if (fwd) wi = wi == 0.0 ? 0.0 : -wi;
                    fc_mul(wr, wi, y[0], y[1], &pr, &pi);
                    accr = accr + pr;
                    acci = acci + pi;
               }
               out[2 * k] = accr;
               out[2 * k + 1] = acci;
          }
          free(ys);
     }
}

static int prime_factors(long n, int *fs)
{
     int c = 0;
     long d = 2;
     while (n > 1) {
          if (d * d > n) { fs[c++] = (int) n; break; }
          if (n % d == 0) { fs[c++] = (int) d; n /= d; }
          else ++d;
     }
     return c;
}

/* Generic-engine 1-D complex DFT of size n on `batch` lines: line b reads
 * in[2*(b*idist + j*istride)] and writes out[2*(b*odist + k*ostride)]. */
int lfo_generic_dft(int fwd, long n, const double *tab, const double *in, long istride,
                    long idist, double *out, long ostride, long odist, long batch, int nthreads)
{
     int fs[64];
     int nf = prime_factors(n, fs);
     long b;
     if (nthreads < 1) nthreads = 1;
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 1)
     for (b = 0; b < batch; ++b) {
          double *o = (double *) malloc(sizeof(double) * 2 * (size_t) n);
          long k;
          gen_exec(fwd, fs, nf, in + 2 * idist * b, istride, o, tab, n);
          for (k = 0; k < n; ++k) {
               out[2 * (odist * b + ostride * k)] = o[2 * k];
               out[2 * (odist * b + ostride * k) + 1] = o[2 * k + 1];
          }
          free(o);
     }
     return 0;
}

/* ------------------------------------------------------------------ 3. double-double DFT */

typedef struct { double hi, lo; } dd;

static inline dd two_sum(double a, double b)
{
     double s = a + b, bb = s - a;
     dd r = { s, (a - (s - bb)) + (b - bb) };
     return r;
}

static inline dd quick_two_sum(double a, double b)
{
     double s = a + b;
     dd r = { s, b - (s - a) };
     return r;
}

static inline dd dd_add(dd a, dd b)
{
     dd s = two_sum(a.hi, b.hi), t = two_sum(a.lo, b.lo);
     s.lo += t.hi;
     s = quick_two_sum(s.hi, s.lo);
     s.lo += t.lo;
     return quick_two_sum(s.hi, s.lo);
}

static inline dd dd_mul(dd a, dd b)
{
     double p = a.hi * b.hi;
     double e = fma(a.hi, b.hi, -p);
     e += a.hi * b.lo + a.lo * b.hi;
     return quick_two_sum(p, e);
}

static inline dd dd_neg(dd a) { dd r = { -a.hi, -a.lo }; return r; }

typedef struct { dd re, im; } cdd;

static inline cdd cdd_add(cdd a, cdd b) { cdd r = { dd_add(a.re, b.re), dd_add(a.im, b.im) }; return r; }
static inline cdd cdd_mul(cdd a, cdd b)
{
     cdd r = { dd_add(dd_mul(a.re, b.re), dd_neg(dd_mul(a.im, b.im))),
               dd_add(dd_mul(a.re, b.im), dd_mul(a.im, b.re)) };
     return r;
}

/* w(m) = exp(sign * 2*pi*i*m/N) from the dd table (cos_hi, cos_lo, sin_hi, sin_lo). */
static inline cdd dd_tw(const double *ddtab, long m, int fwd)
{
     const double *t = ddtab + 4 * m;
     cdd w = { { t[0], t[1] }, { t[2], t[3] } };
     if (fwd) w.im = dd_neg(w.im);
     return w;
}

/* Recursive mixed-radix DIT DFT of size n on x[stride*j]; twiddle exponents are in units of
 * Ntab/n of the table of size Ntab. */
static void dd_fft(int fwd, long n, const cdd *x, long stride, cdd *out, const double *ddtab,
                   long Ntab)
{
     int fs[64];
     int nf = prime_factors(n, fs);
     long k, j;
     if (nf <= 1) {
          for (k = 0; k < n; ++k) {
               cdd acc = { { 0, 0 }, { 0, 0 } };
               for (j = 0; j < n; ++j)
                    acc = cdd_add(acc, cdd_mul(dd_tw(ddtab, (j * k % n) * (Ntab / n), fwd),
                                               x[stride * j]));
               out[k] = acc;
          }
          return;
     }
     {
          int p = fs[0];
          long m = n / p, j1;
          cdd *ys = (cdd *) malloc(sizeof(cdd) * (size_t) n);
          for (j1 = 0; j1 < p; ++j1)
               dd_fft(fwd, m, x + stride * j1, stride * p, ys + m * j1, ddtab, Ntab);
          for (k = 0; k < n; ++k) {
               cdd acc = { { 0, 0 }, { 0, 0 } };
               for (j1 = 0; j1 < p; ++j1)
                    acc = cdd_add(acc, cdd_mul(dd_tw(ddtab, (j1 * k % n) * (Ntab / n), fwd),
                                               ys[m * j1 + k % m]));
               out[k] = acc;
          }
          free(ys);
     }
}

/* Double-double DFT of `batch` lines of size n: line b reads the binary64 pairs
 * in[2*(b*idist + j*istride)] and writes out_hi/out_lo[2*(b*odist + k*ostride)] (+1 for im). */
int lfo_dd_dft(int fwd, long n, const double *ddtab, const double *in, long istride, long idist,
               double *out_hi, double *out_lo, long ostride, long odist, long batch,
               int nthreads)
{
     long b;
     if (nthreads < 1) nthreads = 1;
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 1)
     for (b = 0; b < batch; ++b) {
          cdd *x = (cdd *) malloc(sizeof(cdd) * (size_t) n);
          cdd *y = (cdd *) malloc(sizeof(cdd) * (size_t) n);
          long j;
          for (j = 0; j < n; ++j) {
               const double *p = in + 2 * (idist * b + istride * j);
               x[j].re.hi = p[0]; x[j].re.lo = 0.0;
               x[j].im.hi = p[1]; x[j].im.lo = 0.0;
          }
          dd_fft(fwd, n, x, 1, y, ddtab, n);
          for (j = 0; j < n; ++j) {
               long o = 2 * (odist * b + ostride * j);
               out_hi[o] = y[j].re.hi; out_lo[o] = y[j].re.lo;
               out_hi[o + 1] = y[j].im.hi; out_lo[o + 1] = y[j].im.lo;
          }
          free(x);
          free(y);
     }
     return 0;
}

/* Relative L2 error of y against the double-double reference (hi + lo), over m doubles. */
double lfo_rel_l2(const double *y, const double *ref_hi, const double *ref_lo, long m)
{
     dd num = { 0, 0 }, den = { 0, 0 };
     long i;
     for (i = 0; i < m; ++i) {
          dd r = { ref_hi[i], ref_lo[i] };
          dd d = dd_add(two_sum(y[i], -ref_hi[i]), dd_neg((dd){ ref_lo[i], 0.0 }));
          num = dd_add(num, dd_mul(d, d));
          den = dd_add(den, dd_mul(r, r));
     }
     if (den.hi == 0.0) return num.hi == 0.0 ? 0.0 : INFINITY;
     return sqrt(num.hi / den.hi);
}
