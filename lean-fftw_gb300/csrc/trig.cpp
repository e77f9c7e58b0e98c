// Exact-integer twiddle factors: lean-fftw `LeanFFTW/Core/Trig.lean:25-134` in C++.
//
// Fixed-point numbers are unsigned multiples of 2^-160 held in three 64-bit limbs (every
// value of the series is below 2^162); products use six limbs.  Each step truncates exactly
// where the reference's `Nat` arithmetic does (`fmul` floors, divisions floor), so the
// fixed-point results, and therefore the rounded binary64 values, are identical.
#include "trig.h"

#include <algorithm>
#include <cstring>
#include <thread>

namespace lfg {
namespace {

typedef unsigned __int128 u128;

struct Fx {            // little-endian limbs
  uint64_t w[3];
};

// floor(pi * 10^60) * 2^160 / 10^60, i.e. `piFixed` (Trig.lean:28-33), as limbs.
constexpr Fx kPiFixed = {{0x03707344a4093822ULL, 0x85a308d313198a2eULL, 0x00000003243f6a88ULL}};

inline Fx add(const Fx& a, const Fx& b) {
  Fx r;
  u128 c = 0;
  for (int i = 0; i < 3; ++i) {
    c += (u128)a.w[i] + b.w[i];
    r.w[i] = (uint64_t)c;
    c >>= 64;
  }
  return r;
}

inline Fx sub(const Fx& a, const Fx& b) {  // requires a >= b
  Fx r;
  uint64_t borrow = 0;
  for (int i = 0; i < 3; ++i) {
    u128 d = (u128)a.w[i] - b.w[i] - borrow;
    r.w[i] = (uint64_t)d;
    borrow = (uint64_t)(d >> 127);  // 1 if the subtraction wrapped
  }
  return r;
}

// floor(a*b / 2^160)   (Trig.lean:36)
inline Fx fmul(const Fx& a, const Fx& b) {
  uint64_t p[6] = {0, 0, 0, 0, 0, 0};
  for (int i = 0; i < 3; ++i) {
    u128 c = 0;
    for (int j = 0; j < 3; ++j) {
      c += (u128)a.w[i] * b.w[j] + p[i + j];
      p[i + j] = (uint64_t)c;
      c >>= 64;
    }
    p[i + 3] = (uint64_t)c;
  }
  // shift right by 160 = 2 limbs + 32 bits
  Fx r;
  for (int i = 0; i < 3; ++i) {
    uint64_t lo = p[i + 2] >> 32;
    uint64_t hi = (i + 3 < 6) ? (p[i + 3] << 32) : 0;
    r.w[i] = lo | hi;
  }
  return r;
}

// floor(a / d), d > 0
inline Fx divs(const Fx& a, uint64_t d) {
  Fx r;
  u128 rem = 0;
  for (int i = 2; i >= 0; --i) {
    u128 cur = (rem << 64) | a.w[i];
    r.w[i] = (uint64_t)(cur / d);
    rem = cur % d;
  }
  return r;
}

inline bool is_zero(const Fx& a) { return (a.w[0] | a.w[1] | a.w[2]) == 0; }

inline int bit_length(const Fx& a) {
  for (int i = 2; i >= 0; --i)
    if (a.w[i]) return 64 * i + 64 - __builtin_clzll(a.w[i]);
  return 0;
}

inline int bit(const Fx& a, int i) { return (int)((a.w[i >> 6] >> (i & 63)) & 1); }

inline bool any_below(const Fx& a, int nbits) {  // any of bits [0, nbits) set
  for (int i = 0; i < nbits; ++i)
    if (bit(a, i)) return true;
  return false;
}

// theta * 2^160 for theta = 2*pi*num/den   (Trig.lean:39)
inline Fx angle_fixed(uint64_t num, uint64_t den) {
  // piFixed < 2^162, so 2*piFixed*num < 2^(163 + bits(num)): a 4-limb accumulator.
  uint64_t p[4] = {0, 0, 0, 0};
  Fx twopi = add(kPiFixed, kPiFixed);
  u128 c = 0;
  for (int i = 0; i < 3; ++i) {
    c += (u128)twopi.w[i] * num;
    p[i] = (uint64_t)c;
    c >>= 64;
  }
  p[3] = (uint64_t)c;
  Fx r;
  u128 rem = 0;
  uint64_t q[4];
  for (int i = 3; i >= 0; --i) {
    u128 cur = (rem << 64) | p[i];
    q[i] = (uint64_t)(cur / den);
    rem = cur % den;
  }
  r.w[0] = q[0];
  r.w[1] = q[1];
  r.w[2] = q[2];  // the quotient is <= 2^160 * pi/4
  return r;
}

// Taylor series for cos and sin, 0 <= theta <= pi/4   (Trig.lean:43-62)
void cos_sin_fixed(const Fx& theta, Fx* cos_out, Fx* sin_out) {
  Fx ONE = {{0, 0, 1ULL << 32}};  // 2^160
  Fx th2 = fmul(theta, theta);
  Fx c_pos = ONE, c_neg = {{0, 0, 0}}, s_pos = theta, s_neg = {{0, 0, 0}};
  Fx tc = ONE, ts = theta;
  for (uint64_t j = 1; j < 40; ++j) {
    tc = divs(fmul(tc, th2), (2 * j - 1) * (2 * j));
    ts = divs(fmul(ts, th2), (2 * j) * (2 * j + 1));
    // once both terms are zero every later term is zero too: stopping adds nothing
    if (is_zero(tc) && is_zero(ts)) break;
    if (j % 2 == 1) {
      c_neg = add(c_neg, tc);
      s_neg = add(s_neg, ts);
    } else {
      c_pos = add(c_pos, tc);
      s_pos = add(s_pos, ts);
    }
  }
  *cos_out = sub(c_pos, c_neg);
  *sin_out = sub(s_pos, s_neg);
}

// Round v * 2^-160 (v >= 0) to binary64, ties to even   (Trig.lean:67-86)
double fixed_to_float(const Fx& v) {
  if (is_zero(v)) return 0.0;
  int lg = bit_length(v) - 1;
  uint64_t q;
  if (lg <= 52) {
    q = v.w[0] << (52 - lg);
  } else {
    int sh = lg - 52;
    // q = v >> sh (53 bits)
    q = 0;
    for (int i = 0; i < 53; ++i) q |= (uint64_t)bit(v, sh + i) << i;
    int half_bit = bit(v, sh - 1);
    bool rest = any_below(v, sh - 1);
    if (half_bit && (rest || (q & 1))) q += 1;
  }
  if (q == (1ULL << 53)) {
    q = 1ULL << 52;
    lg += 1;
  }
  uint64_t e = (uint64_t)(lg - 160 + 1023);
  uint64_t bits = (e << 52) | (q - (1ULL << 52));
  double d;
  std::memcpy(&d, &bits, sizeof d);
  return d;
}

inline double neg_z(double x) { return x == 0.0 ? 0.0 : -x; }   // Trig.lean:95

// (cos, sin) of 2*pi*num/(8n), 0 <= num <= n   (Trig.lean:98-100)
void small_at(uint64_t n, uint64_t num, double* c, double* s) {
  Fx cf, sf;
  cos_sin_fixed(angle_fixed(num, 8 * n), &cf, &sf);
  *c = fixed_to_float(cf);
  *s = fixed_to_float(sf);
}

// Exact octant reduction (Trig.lean:104-122), with `small` given as a lookup.
template <class Small>
void octant(uint64_t k, uint64_t n, Small small, double* co, double* so) {
  if (n == 0) {
    *co = 1.0;
    *so = 0.0;
    return;
  }
  k %= n;
  u128 k8 = (u128)8 * k;
  uint64_t oct = (uint64_t)(k8 / n), rem = (uint64_t)(k8 % n);
  double c, s;
  if (oct % 2 == 0) small(rem, &c, &s); else small(n - rem, &c, &s);
  switch (oct) {
    case 0: *co = c; *so = s; break;
    case 1: *co = s; *so = c; break;
    case 2: *co = neg_z(s); *so = c; break;
    case 3: *co = neg_z(c); *so = s; break;
    case 4: *co = neg_z(c); *so = neg_z(s); break;
    case 5: *co = neg_z(s); *so = neg_z(c); break;
    case 6: *co = s; *so = neg_z(c); break;
    default: *co = c; *so = neg_z(s); break;
  }
}

uint64_t gcd64(uint64_t a, uint64_t b) {
  while (b) {
    uint64_t t = a % b;
    a = b;
    b = t;
  }
  return a;
}

}  // namespace

void cos_sin_2pi(uint64_t k, uint64_t n, double* c, double* s) {
  octant(k, n, [n](uint64_t num, double* cc, double* ss) { small_at(n, num, cc, ss); }, c, s);
}

std::vector<double> cos_sin_2pi_table(uint64_t n) {
  std::vector<double> out(2 * n);
  if (n == 0) return out;
  uint64_t g = gcd64(8, n);
  const uint64_t nm = n / g + 1;
  std::vector<double> memo(2 * nm);
  // the series of different angles are independent: spread large tables over host threads
  unsigned nt = std::thread::hardware_concurrency();
  nt = nm < 4096 ? 1 : std::max(1u, std::min(nt, 32u));
  auto work = [&](unsigned id) {
    for (uint64_t i = id; i < nm; i += nt) small_at(n, g * i, &memo[2 * i], &memo[2 * i + 1]);
  };
  if (nt == 1) {
    work(0);
  } else {
    std::vector<std::thread> pool;
    for (unsigned t = 0; t < nt; ++t) pool.emplace_back(work, t);
    for (auto& th : pool) th.join();
  }
  auto lookup = [&](uint64_t num, double* cc, double* ss) {
    *cc = memo[2 * (num / g)];
    *ss = memo[2 * (num / g) + 1];
  };
  for (uint64_t m = 0; m < n; ++m) octant(m, n, lookup, &out[2 * m], &out[2 * m + 1]);
  return out;
}

void pass_twiddles(const std::vector<double>& tab, bool fwd, uint64_t N, int R, uint64_t ns,
                   double* out) {
  uint64_t step = N / (ns * (uint64_t)R);
  size_t o = 0;
  for (int r = 1; r < R; ++r) {
    for (uint64_t k = 0; k < ns; ++k) out[o++] = tab[2 * ((uint64_t)r * k * step)];
    for (uint64_t k = 0; k < ns; ++k) {
      double s = tab[2 * ((uint64_t)r * k * step) + 1];
      out[o++] = fwd ? neg_z(s) : s;
    }
  }
}

}  // namespace lfg
