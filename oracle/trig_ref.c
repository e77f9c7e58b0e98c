/* ORACLE (test infrastructure only): exact-integer cos/sin tables in C.
 *
 * The checker's C restatement of lean-fftw `LeanFFTW/Core/Trig.lean:25-134`, written apart
 * from the product's copy (csrc/trig.cpp): fixed-point values are little-endian arrays of
 * 32-bit limbs (six limbs = 192 bits), multiplied by schoolbook with 64-bit accumulators.
 * Same truncations as the reference (`fmul` floors, divisions floor), same rounding to
 * binary64 (nearest, ties to even).  trig_ref.py checks it against the Python restatement
 * and against the reference's published constants.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define L 6 /* limbs of a fixed-point value (192 bits, values < 2^163) */

typedef struct { uint32_t w[L]; } fx;

/* floor(pi * 10^60) * 2^160 / 10^60 (Trig.lean:28-33): 0x3243f6a8885a308d313198a2e03707344a4093822 */
static const fx PI_FIXED = { { 0xa4093822u, 0x03707344u, 0x13198a2eu, 0x85a308d3u, 0x243f6a88u, 0x3u } };

static void fx_add(fx *r, const fx *a, const fx *b)
{
     uint64_t c = 0;
     for (int i = 0; i < L; ++i) {
          c += (uint64_t) a->w[i] + b->w[i];
          r->w[i] = (uint32_t) c;
          c >>= 32;
     }
}

static void fx_sub(fx *r, const fx *a, const fx *b) /* a >= b */
{
     int64_t br = 0;
     for (int i = 0; i < L; ++i) {
          int64_t d = (int64_t) a->w[i] - b->w[i] - br;
          br = d < 0;
          r->w[i] = (uint32_t) (d + (br << 32));
     }
}

/* floor(a*b / 2^160): 160 bits = 5 limbs */
static void fx_mul(fx *r, const fx *a, const fx *b)
{
     uint32_t p[2 * L];
     memset(p, 0, sizeof p);
     for (int i = 0; i < L; ++i) {
          uint64_t c = 0;
          for (int j = 0; j < L; ++j) {
               c += (uint64_t) a->w[i] * b->w[j] + p[i + j];
               p[i + j] = (uint32_t) c;
               c >>= 32;
          }
          p[i + L] = (uint32_t) c;
     }
     for (int i = 0; i < L; ++i) r->w[i] = p[i + 5];
}

static void fx_div(fx *r, const fx *a, uint32_t d) /* floor(a/d) */
{
     uint64_t rem = 0;
     for (int i = L - 1; i >= 0; --i) {
          uint64_t cur = (rem << 32) | a->w[i];
          r->w[i] = (uint32_t) (cur / d);
          rem = cur % d;
     }
}

/* theta * 2^160 for theta = 2*pi*num/den (Trig.lean:39); den < 2^62 */
static void angle(fx *r, uint64_t num, uint64_t den)
{
     /* 2*piFixed*num in 8 limbs, then long division by den (64-bit) */
     uint32_t p[L + 2];
     uint64_t c = 0;
     fx two;
     fx_add(&two, &PI_FIXED, &PI_FIXED);
     memset(p, 0, sizeof p);
     for (int i = 0; i < L; ++i) {
          unsigned __int128 t = (unsigned __int128) two.w[i] * num + c;
          p[i] = (uint32_t) t;
          c = (uint64_t) (t >> 32);
     }
     p[L] = (uint32_t) c;
     p[L + 1] = (uint32_t) (c >> 32);
     unsigned __int128 rem = 0;
     uint32_t q[L + 2];
     for (int i = L + 1; i >= 0; --i) {
          unsigned __int128 cur = (rem << 32) | p[i];
          q[i] = (uint32_t) (cur / den);
          rem = cur % den;
     }
     for (int i = 0; i < L; ++i) r->w[i] = q[i];
}

static int fx_zero(const fx *a)
{
     for (int i = 0; i < L; ++i) if (a->w[i]) return 0;
     return 1;
}

/* Trig.lean:43-62 (up to 39 terms; the loop stops once both terms are zero, which
 * leaves the sums unchanged) */
static void series(const fx *th, fx *co, fx *si)
{
     fx one = { { 0, 0, 0, 0, 0, 1 } }; /* 2^160 */
     fx t2, cp = one, cn = { { 0 } }, sp = *th, sn = { { 0 } }, tc = one, ts = *th, tmp;
     fx_mul(&t2, th, th);
     for (uint32_t j = 1; j < 40; ++j) {
          fx_mul(&tmp, &tc, &t2);
          fx_div(&tc, &tmp, (2 * j - 1) * (2 * j));
          fx_mul(&tmp, &ts, &t2);
          fx_div(&ts, &tmp, (2 * j) * (2 * j + 1));
          if (fx_zero(&tc) && fx_zero(&ts)) break; /* later terms are all zero */
          if (j & 1) { fx_add(&cn, &cn, &tc); fx_add(&sn, &sn, &ts); }
          else { fx_add(&cp, &cp, &tc); fx_add(&sp, &sp, &ts); }
     }
     fx_sub(co, &cp, &cn);
     fx_sub(si, &sp, &sn);
}

static int fx_bit(const fx *a, int i) { return (a->w[i >> 5] >> (i & 31)) & 1; }

/* Trig.lean:67-86 */
static double to_double(const fx *v)
{
     int lg = -1;
     uint64_t q = 0, bits;
     double d;
     if (fx_zero(v)) return 0.0;
     for (int i = 32 * L - 1; i >= 0; --i) if (fx_bit(v, i)) { lg = i; break; }
     if (lg <= 52) {
          for (int i = 0; i <= lg; ++i) q |= (uint64_t) fx_bit(v, i) << (i + 52 - lg);
     } else {
          int sh = lg - 52, rest = 0;
          for (int i = 0; i < 53; ++i) q |= (uint64_t) fx_bit(v, sh + i) << i;
          for (int i = 0; i < sh - 1; ++i) rest |= fx_bit(v, i);
          if (fx_bit(v, sh - 1) && (rest || (q & 1))) q += 1;
     }
     if (q == (1ULL << 53)) { q = 1ULL << 52; lg += 1; }
     bits = ((uint64_t) (lg - 160 + 1023) << 52) | (q - (1ULL << 52));
     memcpy(&d, &bits, sizeof d);
     return d;
}

static double nz(double x) { return x == 0.0 ? 0.0 : -x; }

/* out[2m], out[2m+1] = cos, sin (2*pi*m/n), m < n (Trig.lean:104-134): the reduced angles
 * are multiples of g = gcd(8, n), so n/g + 1 series are summed. */
int lfo_cos_sin_table(uint64_t n, double *out)
{
     uint64_t g = 8, a = n;
     while (a) { uint64_t t = g % a; g = a; a = t; }
     uint64_t nm = n / g + 1;
     double *memo = (double *) malloc(sizeof(double) * 2 * nm);
     if (!memo) return -1;
#pragma omp parallel for schedule(static) if (nm > 4096)
     for (uint64_t i = 0; i < nm; ++i) {
          fx th, cf, sf;
          angle(&th, g * i, 8 * n);
          series(&th, &cf, &sf);
          memo[2 * i] = to_double(&cf);
          memo[2 * i + 1] = to_double(&sf);
     }
     for (uint64_t m = 0; m < n; ++m) {
          unsigned __int128 k8 = (unsigned __int128) 8 * m;
          uint64_t oct = (uint64_t) (k8 / n), rem = (uint64_t) (k8 % n);
          uint64_t num = (oct % 2 == 0) ? rem : n - rem;
          double c = memo[2 * (num / g)], s = memo[2 * (num / g) + 1];
          switch (oct) {
          case 0: out[2 * m] = c; out[2 * m + 1] = s; break;
          case 1: out[2 * m] = s; out[2 * m + 1] = c; break;
          case 2: out[2 * m] = nz(s); out[2 * m + 1] = c; break;
          case 3: out[2 * m] = nz(c); out[2 * m + 1] = s; break;
          case 4: out[2 * m] = nz(c); out[2 * m + 1] = nz(s); break;
          case 5: out[2 * m] = nz(s); out[2 * m + 1] = nz(c); break;
          case 6: out[2 * m] = s; out[2 * m + 1] = nz(c); break;
          default: out[2 * m] = c; out[2 * m + 1] = nz(s); break;
          }
     }
     free(memo);
     return 0;
}
