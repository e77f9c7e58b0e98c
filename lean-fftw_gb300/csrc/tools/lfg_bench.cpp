// lfg-bench: a libbench2-style command line over the library's C ABI, so that lean-fftw's
// benchmark driver (tools/bench.py: `-s <problem>` for speed, `-v1 --verify <problem>` for
// accuracy) can run the GPU engine as one more implementation.
//
//   lfg-bench -s <problem>         Problem: <p>, setup: <t>, time: <t>, ``mflops'': <x>
//   lfg-bench --verify <problem>   <p> <linearity error> <impulse error> <shift error>
//   lfg-bench --can-do <problem>   #t or #f
//   lfg-bench --parse <problem>    the FFI spec the problem maps to (no GPU needed)
//   options: -o device (time device-resident buffers instead of host buffers),
//            -t <seconds> (minimum timed interval, default 0.01), --print-precision, -v<n>
//
// Problem strings follow FFTW's libbench2 grammar (as classified by lean-fftw
// tools/classify_problems.py:7-40): flags [i|o][/][f|b|-|+][c|r|k], dimensions n1xn2x...,
// each optionally n:is:os, then an optional vector `*m1xm2...` (vector outermost) or
// `v m1x...` (vector innermost).  Default strides are row-major; rdft2 problems keep the
// real side's last dimension n (out of place) or 2(n/2+1) (in place) and the complex side's
// n/2+1.  The problem becomes lean-fftw's FFI spec (LeanFFTW/FFI.lean:13-21, strides in
// doubles) and goes to lfg_plan_spec; what the library does not execute is `#f`.
//
// Speed follows the libbench2 protocol: the iteration count doubles until one timing covers
// at least the minimum interval, then the best of 8 timings is reported per transform.  The
// default times lfg_execute_host on pinned host arrays (the lfa_call contract).
//
// Verification is the randomized test of FFTW's verifier (after F. Ergun, "Testing
// multivariate linear functions", STOC 1995): linearity F(a x + b y) = a F(x) + b F(y), the
// impulse response F(delta + r) - F(r) = 1, and the time shift of one sample along each
// dimension, which multiplies the spectrum by exp(sign 2 pi i k_d / n_d).  Each error is a
// relative L2 norm; phase factors come from the library's exact cos/sin table.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "lfg.h"

namespace {

using cplx = std::complex<double>;

struct Dim {
  int64_t n = 1, is = 0, os = 0;
  bool strided = false;
  int r2r = -1;  // r2r kind of the dimension (libbench2 numbering); -1: none given
};

struct Problem {
  std::string text;
  bool inplace = false, split = false;
  int sign = -1;
  char kind = 'c';
  std::vector<Dim> sz, vec;
  bool vec_inner = false;
  std::string err;
};

bool parse_dims(const std::string& t, std::vector<Dim>* out, std::string* err) {
  size_t i = 0;
  while (i < t.size()) {
    size_t j = t.find('x', i);
    if (j == std::string::npos) j = t.size();
    std::string d = t.substr(i, j - i);
    Dim dm;
    size_t k = 0;
    auto num = [&](int64_t* v) -> bool {
      size_t s = k;
      if (k < d.size() && d[k] == '-') ++k;
      while (k < d.size() && isdigit((unsigned char)d[k])) ++k;
      if (k == s || (k == s + 1 && d[s] == '-')) return false;
      *v = std::strtoll(d.substr(s, k - s).c_str(), nullptr, 10);
      return true;
    };
    if (!num(&dm.n)) { *err = "bad dimension '" + d + "'"; return false; }
    if (k < d.size() && d[k] == ':') {
      ++k;
      if (!num(&dm.is)) { *err = "bad stride in '" + d + "'"; return false; }
      dm.os = dm.is;
      if (k < d.size() && d[k] == ':') {
        ++k;
        if (!num(&dm.os)) { *err = "bad stride in '" + d + "'"; return false; }
      }
      dm.strided = true;
    }
    if (k < d.size()) {   // r2r kind suffix: f b h (R2HC HC2R DHT), e00..e11, o00..o11
      const char c = (char)tolower((unsigned char)d[k]);
      if (c == 'f' || c == 'b' || c == 'h') {
        dm.r2r = c == 'f' ? 0 : c == 'b' ? 1 : 2;
        ++k;
      } else if ((c == 'e' || c == 'o') && k + 3 == d.size() &&
                 (d[k + 1] == '0' || d[k + 1] == '1') && (d[k + 2] == '0' || d[k + 2] == '1')) {
        const int code = (d[k + 1] - '0') * 2 + (d[k + 2] - '0');   // 00 01 10 11
        dm.r2r = (c == 'e' ? 3 : 7) + code;
        k += 3;
      }
    }
    if (k != d.size()) { *err = "bad dimension suffix in '" + d + "'"; return false; }
    out->push_back(dm);
    i = j + 1;
  }
  return true;
}

Problem parse(const std::string& s) {
  Problem p;
  p.text = s;
  size_t i = 0;
  for (; i < s.size(); ++i) {
    const char c = (char)tolower((unsigned char)s[i]);
    if (c == 'i') p.inplace = true;
    else if (c == 'o') p.inplace = false;
    else if (c == 'd') {}
    else if (c == '/') p.split = true;
    else if (c == 'f' || c == '-') p.sign = -1;
    else if (c == 'b' || c == '+') p.sign = 1;
    else if (c == 'r' || c == 'c' || c == 'k') p.kind = c;
    else break;
  }
  std::string rest = s.substr(i), vec;
  const size_t star = rest.find_first_of("*vV");
  if (star != std::string::npos) {
    p.vec_inner = rest[star] != '*';
    vec = rest.substr(star + 1);
    rest = rest.substr(0, star);
  }
  if (rest.empty()) p.err = "no transform dimensions";
  else if (parse_dims(rest, &p.sz, &p.err) && !vec.empty()) parse_dims(vec, &p.vec, &p.err);
  if (p.err.empty() && p.split && p.kind == 'k') p.err = "r2r problems have no split arrays";
  // an r2r dimension without a kind suffix is R2HC forward, HC2R backward; other problems
  // take no kind suffixes
  for (Dim& d : p.sz) {
    if (p.kind != 'k' && d.r2r >= 0 && p.err.empty()) p.err = "r2r kind suffix on a non-r2r problem";
    if (d.r2r < 0) d.r2r = p.sign < 0 ? 0 : 1;
  }
  for (const Dim& d : p.vec)
    if (d.r2r >= 0 && p.err.empty()) p.err = "kind suffix on a vector dimension";
  return p;
}

// Row-major default strides of `dims` (phys: physical extents) times `mul`.
void rowmajor(std::vector<Dim>& dims, const std::vector<int64_t>& phys, int64_t mul, bool in_side) {
  int64_t acc = mul;
  for (int d = (int)dims.size() - 1; d >= 0; --d) {
    if (!dims[d].strided) (in_side ? dims[d].is : dims[d].os) = acc;
    acc *= phys[d];
  }
}

int64_t prod(const std::vector<int64_t>& v) {
  int64_t p = 1;
  for (int64_t x : v) p *= x;
  return p;
}

// Layout of a problem: strides of every dimension on both sides (elements of each side:
// complex values, or real scalars on the real side of rdft2), and the spec for lfg_plan_spec.
struct Layout {
  std::vector<Dim> sz, vec;
  bool in_real = false, out_real = false;
  int64_t in_lo = 0, in_hi = 0, out_lo = 0, out_hi = 0;   // element offset ranges
  // element o of a side (offset relative to the low end of its span) has its real part at
  // double re + mult * o and its imaginary part at im + mult * o (interleaved: im = re + 1,
  // mult 2; split arrays: the imaginary array follows the real one, mult 1)
  int64_t in_re = 0, in_im = 0, out_re = 0, out_im = 0, in_mult = 2, out_mult = 2;
  int64_t in_len = 0, out_len = 0;   // doubles of each buffer
  std::vector<double> spec;
};

void span(const std::vector<Dim>& all, bool out, int64_t last_half_rank, int64_t* lo, int64_t* hi) {
  *lo = *hi = 0;
  for (size_t i = 0; i < all.size(); ++i) {
    int64_t n = all[i].n;
    if ((int64_t)i == last_half_rank) n = n / 2 + 1;
    const int64_t s = out ? all[i].os : all[i].is;
    if (n > 1) {
      if (s > 0) *hi += (n - 1) * s;
      else *lo += (n - 1) * s;
    }
  }
}

Layout layout(const Problem& p) {
  Layout L;
  L.sz = p.sz;
  L.vec = p.vec;
  const int r = (int)p.sz.size();
  const bool real = p.kind == 'r', r2r = p.kind == 'k';
  L.in_real = (real && p.sign < 0) || r2r;
  L.out_real = (real && p.sign > 0) || r2r;
  std::vector<int64_t> vphys;
  for (const Dim& d : p.vec) vphys.push_back(d.n);
  const int64_t V = prod(vphys);
  for (int side = 0; side < 2; ++side) {   // 0: input, 1: output
    const bool is_real = side == 0 ? L.in_real : L.out_real;
    std::vector<int64_t> phys;
    for (const Dim& d : p.sz) phys.push_back(d.n);
    if (real) {
      const int64_t nl = p.sz[r - 1].n;
      phys[r - 1] = is_real ? (p.inplace ? 2 * (nl / 2 + 1) : nl) : nl / 2 + 1;
    }
    const int64_t S = prod(phys);
    rowmajor(L.sz, phys, p.vec_inner ? V : 1, side == 0);
    rowmajor(L.vec, vphys, p.vec_inner ? 1 : S, side == 0);
  }
  std::vector<Dim> all = L.sz;
  all.insert(all.end(), L.vec.begin(), L.vec.end());
  span(all, false, (real && !L.in_real) ? r - 1 : -1, &L.in_lo, &L.in_hi);
  span(all, true, (real && !L.out_real) ? r - 1 : -1, &L.out_lo, &L.out_hi);
  // spec: strides and offsets in doubles; buffers start at the low end of each span
  const int64_t in_span = L.in_hi - L.in_lo + 1, out_span = L.out_hi - L.out_lo + 1;
  const int64_t span_both = std::max(in_span, out_span);
  auto side = [&](bool is_real, int64_t lo, int64_t span, int64_t* re, int64_t* imb, int64_t* mult,
                  int64_t* len) {
    if (is_real) {
      *mult = 1;
      *re = -lo;
      *imb = *re;
      *len = span;
    } else if (p.split) {
      *mult = 1;
      *re = -lo;
      *imb = *re + (p.inplace ? span_both : span);
      *len = 2 * (p.inplace ? span_both : span);
    } else {
      *mult = 2;
      *re = -2 * lo;
      *imb = *re + 1;
      *len = 2 * span;
    }
  };
  side(L.in_real, L.in_lo, in_span, &L.in_re, &L.in_im, &L.in_mult, &L.in_len);
  side(L.out_real, L.out_lo, out_span, &L.out_re, &L.out_im, &L.out_mult, &L.out_len);
  const double im = (double)L.in_mult, om = (double)L.out_mult;
  L.spec = {r2r ? 2.0 : real ? 1.0 : 0.0, (double)p.sign, (double)r, (double)p.vec.size(),
            (double)L.in_re, (double)L.in_im, (double)L.out_re, (double)L.out_im};
  for (const Dim& d : L.sz) {
    L.spec.push_back((double)d.n);
    L.spec.push_back(d.is * im);
    L.spec.push_back(d.os * om);
  }
  for (const Dim& d : L.vec) {
    L.spec.push_back((double)d.n);
    L.spec.push_back(d.is * im);
    L.spec.push_back(d.os * om);
  }
  if (r2r)
    for (const Dim& d : L.sz) L.spec.push_back((double)d.r2r);
  return L;
}

// doubles each side's buffer holds
int64_t in_doubles(const Layout& L, bool inplace) {
  return inplace ? std::max(L.in_len, L.out_len) + 2 : L.in_len;
}
int64_t out_doubles(const Layout& L) { return L.out_len; }

struct Runner {
  Problem p;
  Layout L;
  lfg_plan* plan = nullptr;
  double* hin = nullptr;
  double* hout = nullptr;
  int64_t nin = 0, nout = 0;
  bool device = false;
  void* din = nullptr;
  void* dout = nullptr;

  std::string setup() {
    lfg_status s = lfg_plan_spec(L.spec.data(), L.spec.size(), LFG_F64, LFG_ESTIMATE, &plan);
    if (s != LFG_OK) return lfg_last_error();
    nin = in_doubles(L, p.inplace);
    nout = p.inplace ? nin : out_doubles(L);
    if (cudaMallocHost((void**)&hin, nin * 8) != cudaSuccess) return "cudaMallocHost failed";
    hout = hin;
    if (!p.inplace && cudaMallocHost((void**)&hout, nout * 8) != cudaSuccess) return "cudaMallocHost failed";
    std::memset(hin, 0, nin * 8);
    if (!p.inplace) std::memset(hout, 0, nout * 8);
    if (device) {
      if (cudaMalloc(&din, nin * 8) != cudaSuccess) return "cudaMalloc failed";
      dout = din;
      if (!p.inplace && cudaMalloc(&dout, nout * 8) != cudaSuccess) return "cudaMalloc failed";
      cudaMemset(din, 0, nin * 8);
      if (!p.inplace) cudaMemset(dout, 0, nout * 8);
    }
    return "";
  }
  bool exec() {
    if (device) return lfg_execute(plan, din, dout, nullptr) == LFG_OK;
    return lfg_execute_host(plan, hin, hout) == LFG_OK;
  }
  ~Runner() {
    if (plan) lfg_destroy(plan);
    if (hout && hout != hin) cudaFreeHost(hout);
    if (hin) cudaFreeHost(hin);
    if (dout && dout != din) cudaFree(dout);
    if (din) cudaFree(din);
  }

  // ---- logical access: index = (vector indices, transform indices), row-major ----
  int64_t count(bool out_side, bool halved) const {
    int64_t c = 1;
    for (size_t d = 0; d < L.vec.size(); ++d) c *= L.vec[d].n;
    for (size_t d = 0; d < L.sz.size(); ++d)
      c *= (halved && d + 1 == L.sz.size()) ? L.sz[d].n / 2 + 1 : L.sz[d].n;
    (void)out_side;
    return c;
  }
  // element offset (in side elements, relative to the buffer start) of logical index q
  int64_t offset(int64_t q, bool out_side, bool halved) const {
    int64_t off = 0;
    for (int d = (int)L.sz.size() - 1; d >= 0; --d) {
      const int64_t n = (halved && d + 1 == (int)L.sz.size()) ? L.sz[d].n / 2 + 1 : L.sz[d].n;
      off += (q % n) * (out_side ? L.sz[d].os : L.sz[d].is);
      q /= n;
    }
    for (int d = (int)L.vec.size() - 1; d >= 0; --d) {
      const int64_t n = L.vec[d].n;
      off += (q % n) * (out_side ? L.vec[d].os : L.vec[d].is);
      q /= n;
    }
    return off - (out_side ? L.out_lo : L.in_lo);
  }
  // run on a logical input (complex values; real sides use the real parts)
  std::vector<cplx> run(const std::vector<cplx>& x) {
    const bool ih = p.kind == 'r' && !L.in_real, oh = p.kind == 'r' && !L.out_real;
    std::memset(hin, 0, nin * 8);
    for (int64_t q = 0; q < (int64_t)x.size(); ++q) {
      const int64_t o = offset(q, false, ih);
      hin[L.in_re + L.in_mult * o] = x[q].real();
      if (!L.in_real) hin[L.in_im + L.in_mult * o] = x[q].imag();
    }
    if (device) {
      cudaMemcpy(din, hin, nin * 8, cudaMemcpyHostToDevice);
      exec();
      cudaMemcpy(hout, dout, nout * 8, cudaMemcpyDeviceToHost);
    } else {
      exec();
    }
    std::vector<cplx> y(count(true, oh));
    for (int64_t q = 0; q < (int64_t)y.size(); ++q) {
      const int64_t o = offset(q, true, oh);
      y[q] = L.out_real ? cplx(hout[L.out_re + o], 0.0)
                        : cplx(hout[L.out_re + L.out_mult * o], hout[L.out_im + L.out_mult * o]);
    }
    return y;
  }
};

std::string fmt_time(double t) {
  char b[64];
  if (t < 1e-6) std::snprintf(b, sizeof b, "%.2f ns", t * 1e9);
  else if (t < 1e-3) std::snprintf(b, sizeof b, "%.2f us", t * 1e6);
  else if (t < 1.0) std::snprintf(b, sizeof b, "%.2f ms", t * 1e3);
  else std::snprintf(b, sizeof b, "%.2f s", t);
  return b;
}

double now() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

int speed(Runner& R, double tmin) {
  const double t0 = now();
  std::string e = R.setup();
  if (!e.empty()) { std::fprintf(stderr, "lfg-bench: %s\n", e.c_str()); return 1; }
  if (!R.exec()) { std::fprintf(stderr, "lfg-bench: %s\n", lfg_last_error()); return 1; }
  if (R.device) cudaDeviceSynchronize();
  const double setup = now() - t0;
  auto timed = [&](int64_t iters) {
    if (R.device) cudaDeviceSynchronize();
    const double a = now();
    for (int64_t i = 0; i < iters; ++i) R.exec();
    if (R.device) cudaDeviceSynchronize();
    return now() - a;
  };
  int64_t iters = 1;
  while (timed(iters) < tmin && iters < ((int64_t)1 << 40)) iters *= 2;
  double best = 1e300;
  for (int k = 0; k < 8; ++k) best = std::min(best, timed(iters) / (double)iters);
  double n = 1, howmany = 1;
  for (const Dim& d : R.p.sz) n *= (double)d.n;
  for (const Dim& d : R.p.vec) howmany *= (double)d.n;
  const double flops = (R.p.kind == 'c' ? 5.0 : 2.5) * n * std::log2(std::max(n, 2.0)) * howmany;
  std::printf("Problem: %s, setup: %s, time: %s, ``mflops'': %.5g\n", R.p.text.c_str(),
              fmt_time(setup).c_str(), fmt_time(best).c_str(), flops / best / 1e6);
  return 0;
}

double rel_l2(const std::vector<cplx>& a, const std::vector<cplx>& b) {
  double num = 0, den = 0;
  for (size_t i = 0; i < a.size(); ++i) {
    num += std::norm(a[i] - b[i]);
    den += std::norm(b[i]);
  }
  return den > 0 ? std::sqrt(num / den) : std::sqrt(num);
}

// FFTW's definitions of the r2r kinds (unnormalised), evaluated directly in long double:
// y = T x for one line of n values.
void r2r_direct(int kind, int64_t n, const long double* x, long double* y) {
  const long double pi = 3.141592653589793238462643383279502884L;
  for (int64_t k = 0; k < n; ++k) {
    long double s = 0;
    switch (kind) {
      case 0:   // R2HC: r_k at k <= n/2, -sum x sin at n-k
        if (k <= n / 2) {
          for (int64_t j = 0; j < n; ++j) s += x[j] * std::cos(2 * pi * (long double)(j * k % n) / n);
        } else {
          for (int64_t j = 0; j < n; ++j) s -= x[j] * std::sin(2 * pi * (long double)(j * (n - k) % n) / n);
        }
        break;
      case 1:   // HC2R: halfcomplex in, real out
        s = x[0];
        for (int64_t m = 1; m < n - m; ++m)
          s += 2 * (x[m] * std::cos(2 * pi * (long double)(k * m % n) / n) -
                    x[n - m] * std::sin(2 * pi * (long double)(k * m % n) / n));
        if (n % 2 == 0 && n > 1) s += x[n / 2] * ((k % 2) ? -1 : 1);
        break;
      case 2:   // DHT
        for (int64_t j = 0; j < n; ++j) {
          const long double a = 2 * pi * (long double)(j * k % n) / n;
          s += x[j] * (std::cos(a) + std::sin(a));
        }
        break;
      case 3:   // REDFT00
        s = x[0] + ((k % 2) ? -x[n - 1] : x[n - 1]);
        for (int64_t j = 1; j + 1 < n; ++j) s += 2 * x[j] * std::cos(pi * j * k / (long double)(n - 1));
        break;
      case 4:   // REDFT01
        s = x[0];
        for (int64_t j = 1; j < n; ++j) s += 2 * x[j] * std::cos(pi * j * (k + 0.5L) / n);
        break;
      case 5:   // REDFT10
        for (int64_t j = 0; j < n; ++j) s += 2 * x[j] * std::cos(pi * (j + 0.5L) * k / n);
        break;
      case 6:   // REDFT11
        for (int64_t j = 0; j < n; ++j) s += 2 * x[j] * std::cos(pi * (j + 0.5L) * (k + 0.5L) / n);
        break;
      case 7:   // RODFT00
        for (int64_t j = 0; j < n; ++j) s += 2 * x[j] * std::sin(pi * (j + 1) * (k + 1) / (long double)(n + 1));
        break;
      case 8:   // RODFT01
        s = (k % 2) ? -x[n - 1] : x[n - 1];
        for (int64_t j = 0; j + 1 < n; ++j) s += 2 * x[j] * std::sin(pi * (j + 1) * (k + 0.5L) / n);
        break;
      case 9:   // RODFT10
        for (int64_t j = 0; j < n; ++j) s += 2 * x[j] * std::sin(pi * (j + 0.5L) * (k + 1) / n);
        break;
      default:  // RODFT11
        for (int64_t j = 0; j < n; ++j) s += 2 * x[j] * std::sin(pi * (j + 0.5L) * (k + 0.5L) / n);
        break;
    }
    y[k] = s;
  }
}

// r2r verification: linearity, the impulse response and a random input against the direct
// evaluation of the definitions along every axis (long double).
int verify_r2r(Runner& R, int rounds) {
  const Problem& p = R.p;
  const int r = (int)p.sz.size();
  const int nv = (int)p.vec.size();
  std::vector<int64_t> ext;
  for (const Dim& d : p.vec) ext.push_back(d.n);
  for (const Dim& d : p.sz) ext.push_back(d.n);
  const int64_t total = prod(ext);
  std::mt19937_64 gen(20261016);
  std::uniform_real_distribution<double> U(-0.5, 0.5);
  auto direct = [&](const std::vector<cplx>& x) {
    std::vector<long double> a(total);
    for (int64_t i = 0; i < total; ++i) a[i] = x[i].real();
    for (int d = 0; d < r; ++d) {
      const int axis = nv + d;
      const int64_t n = ext[axis];
      int64_t stride = 1;
      for (int i = (int)ext.size() - 1; i > axis; --i) stride *= ext[i];
      std::vector<long double> line(n), out(n);
      for (int64_t base = 0; base < total; ++base) {
        if ((base / stride) % n != 0) continue;   // first element of each line along axis
        for (int64_t j = 0; j < n; ++j) line[j] = a[base + j * stride];
        r2r_direct(p.sz[d].r2r, n, line.data(), out.data());
        for (int64_t j = 0; j < n; ++j) a[base + j * stride] = out[j];
      }
    }
    std::vector<cplx> y(total);
    for (int64_t i = 0; i < total; ++i) y[i] = cplx((double)a[i], 0.0);
    return y;
  };
  double el = 0, ei = 0, er = 0;
  for (int round = 0; round < rounds; ++round) {
    std::vector<cplx> x(total), y(total), z(total);
    for (auto& v : x) v = cplx(U(gen), 0.0);
    for (auto& v : y) v = cplx(U(gen), 0.0);
    const double a = U(gen), b = U(gen);
    for (int64_t i = 0; i < total; ++i) z[i] = a * x[i] + b * y[i];
    const std::vector<cplx> Fx = R.run(x), Fy = R.run(y), Fz = R.run(z);
    std::vector<cplx> lin(total);
    for (int64_t i = 0; i < total; ++i) lin[i] = a * Fx[i] + b * Fy[i];
    el = std::max(el, rel_l2(Fz, lin));
    std::vector<cplx> d(total, cplx(0.0, 0.0));
    const int64_t per = total / std::max<int64_t>(1, prod(std::vector<int64_t>(ext.begin(), ext.begin() + nv)));
    for (int64_t v = 0; v < total; v += per) d[v] = 1.0;
    ei = std::max(ei, rel_l2(R.run(d), direct(d)));
    er = std::max(er, rel_l2(Fx, direct(x)));
  }
  std::printf("%s %.3g %.3g %.3g\n", p.text.c_str(), el, ei, er);
  return 0;
}

int verify(Runner& R, int rounds) {
  if (R.p.kind == 'k') {
    std::string e = R.setup();
    if (!e.empty()) { std::fprintf(stderr, "lfg-bench: %s\n", e.c_str()); return 1; }
    return verify_r2r(R, rounds);
  }
  std::string e = R.setup();
  if (!e.empty()) { std::fprintf(stderr, "lfg-bench: %s\n", e.c_str()); return 1; }
  const Problem& p = R.p;
  const bool real = p.kind == 'r', c2r = real && p.sign > 0;
  const int r = (int)p.sz.size();
  const int64_t nin = R.count(false, real && !R.L.in_real);
  const int64_t nout = R.count(true, real && !R.L.out_real);
  int64_t V = 1;
  for (const Dim& d : p.vec) V *= d.n;
  std::mt19937_64 gen(20261016);
  std::uniform_real_distribution<double> U(-0.5, 0.5);
  // logical input extents (vector dims first, then transform dims; last halved on c2r input)
  std::vector<int64_t> ext;
  for (const Dim& d : p.vec) ext.push_back(d.n);
  for (int d = 0; d < r; ++d) ext.push_back(c2r && d == r - 1 ? p.sz[d].n / 2 + 1 : p.sz[d].n);
  const int nv = (int)p.vec.size();
  auto random_input = [&]() {
    std::vector<cplx> x(nin);
    for (auto& v : x) v = real && !c2r ? cplx(U(gen), 0.0) : cplx(U(gen), U(gen));
    if (c2r) {
      // a Hermitian-consistent half spectrum: self-conjugate columns k_last in {0, n/2}
      const int64_t nl = p.sz[r - 1].n, h = nl / 2 + 1, n0 = r == 2 ? p.sz[0].n : 1;
      for (int64_t b = 0; b < V; ++b)
        for (int64_t kl : {(int64_t)0, nl % 2 == 0 ? nl / 2 : (int64_t)-1}) {
          if (kl < 0) continue;
          for (int64_t k0 = 0; k0 < n0; ++k0) {
            const int64_t k0c = (n0 - k0) % n0;
            cplx& a = x[(b * n0 + k0) * h + kl];
            if (k0c == k0) a = cplx(a.real(), 0.0);
            else if (k0c < k0) a = std::conj(x[(b * n0 + k0c) * h + kl]);
          }
        }
    }
    return x;
  };
  double el = 0, ei = 0, es = 0;
  for (int round = 0; round < rounds; ++round) {
    // linearity (real scalars on the real transforms)
    std::vector<cplx> x = random_input(), y = random_input(), z(nin);
    const cplx a = real ? cplx(U(gen), 0.0) : cplx(U(gen), U(gen));
    const cplx b = real ? cplx(U(gen), 0.0) : cplx(U(gen), U(gen));
    for (int64_t i = 0; i < nin; ++i) z[i] = a * x[i] + b * y[i];
    const std::vector<cplx> Fx = R.run(x), Fy = R.run(y), Fz = R.run(z);
    std::vector<cplx> lin(nout);
    for (int64_t i = 0; i < nout; ++i) lin[i] = a * Fx[i] + b * Fy[i];
    el = std::max(el, rel_l2(Fz, lin));
    // impulse: F(delta + x) - F(x) = 1 everywhere
    std::vector<cplx> d = x;
    const int64_t per = nin / V;
    for (int64_t v = 0; v < V; ++v) d[v * per] += 1.0;
    const std::vector<cplx> Fd = R.run(d);
    std::vector<cplx> diff(nout), ones(nout, cplx(1.0, 0.0));
    for (int64_t i = 0; i < nout; ++i) diff[i] = Fd[i] - Fx[i];
    ei = std::max(ei, rel_l2(diff, ones));
    // one-sample shift along each transform dimension
    for (int dd = 0; dd < r; ++dd) {
      const int64_t nd = p.sz[dd].n;
      std::vector<double> tab(2 * nd);
      lfg_cos_sin_table((uint64_t)nd, tab.data());
      auto w = [&](int64_t k, int sgn) { return cplx(tab[2 * (k % nd)], sgn * tab[2 * (k % nd) + 1]); };
      // strides of the logical arrays
      auto coord = [&](int64_t q, const std::vector<int64_t>& ex, int axis) {
        for (int i = (int)ex.size() - 1; i > axis; --i) q /= ex[i];
        return q % ex[axis];
      };
      const int axis = nv + dd;
      std::vector<int64_t> oext = ext;   // output extents: the halved side is the complex one
      if (real) oext[nv + r - 1] = c2r ? p.sz[r - 1].n : p.sz[r - 1].n / 2 + 1;
      int64_t stride = 1;
      for (int i = (int)ext.size() - 1; i > axis; --i) stride *= ext[i];
      std::vector<cplx> xs(nin), expect(nout);
      if (!c2r) {
        // x'[j] = x[j - e_d]: F(x')[k] = F(x)[k] * exp(sign 2 pi i k_d / n_d)
        for (int64_t q = 0; q < nin; ++q) {
          const int64_t j = coord(q, ext, axis);
          xs[q] = x[q + (((j + nd - 1) % nd) - j) * stride];
        }
        for (int64_t q = 0; q < nout; ++q) expect[q] = Fx[q] * w(coord(q, oext, axis), p.sign);
      } else {
        // H'[k] = H[k] exp(-2 pi i k_d / n_d) shifts the real output by one sample
        for (int64_t q = 0; q < nin; ++q) xs[q] = x[q] * w(coord(q, ext, axis), -1);
        int64_t ostride = 1;
        for (int i = (int)oext.size() - 1; i > axis; --i) ostride *= oext[i];
        for (int64_t q = 0; q < nout; ++q) {
          const int64_t j = coord(q, oext, axis);
          expect[q] = Fx[q + (((j + nd - 1) % nd) - j) * ostride];
        }
      }
      es = std::max(es, rel_l2(R.run(xs), expect));
    }
  }
  std::printf("%s %.3g %.3g %.3g\n", p.text.c_str(), el, ei, es);
  return 0;
}

void usage() {
  std::fprintf(stderr,
               "usage: lfg-bench [-s|--speed P] [-y|--verify P] [-d|--can-do P] [--parse P]\n"
               "                 [-o device] [-t seconds] [-v<n>] [--print-precision]\n");
}

}  // namespace

int main(int argc, char** argv) {
  bool device = false;
  double tmin = 0.01;
  int rounds = 3;
  std::string mode, prob;
  for (int i = 1; i < argc; ++i) {
    std::string a = argv[i];
    auto next = [&]() -> std::string { return i + 1 < argc ? argv[++i] : ""; };
    if (a == "-s" || a == "--speed") { mode = "speed"; prob = next(); }
    else if (a == "-y" || a == "--verify") { mode = "verify"; prob = next(); }
    else if (a == "-d" || a == "--can-do") { mode = "cando"; prob = next(); }
    else if (a == "--parse") { mode = "parse"; prob = next(); }
    else if (a == "-o") { if (next() == "device") device = true; }
    else if (a == "-t") tmin = std::atof(next().c_str());
    else if (a == "-r") rounds = std::max(1, std::atoi(next().c_str()));
    else if (a.rfind("-v", 0) == 0) {}
    else if (a == "--print-precision") { std::printf("double\n"); return 0; }
    else if (a == "--info-all") {
      std::printf("(name \"lean-fftw-gb300\")\n(version \"1\")\n(precision \"double\")\n");
      return 0;
    } else { usage(); return 2; }
  }
  if (mode.empty() || prob.empty()) { usage(); return 2; }
  Problem p = parse(prob);
  if (mode == "parse") {
    if (!p.err.empty()) { std::printf("unsupported: %s\n", p.err.c_str()); return 0; }
    Layout L = layout(p);
    for (size_t i = 0; i < L.spec.size(); ++i) std::printf("%s%g", i ? " " : "", L.spec[i]);
    std::printf("\n");
    return 0;
  }
  if (!p.err.empty()) {
    if (mode == "cando") { std::printf("#f\n"); return 0; }
    std::fprintf(stderr, "lfg-bench: %s\n", p.err.c_str());
    return 1;
  }
  Runner R;
  R.p = p;
  R.L = layout(p);
  R.device = device;
  if (mode == "cando") {
    lfg_plan* h = nullptr;
    const bool ok = lfg_plan_spec(R.L.spec.data(), R.L.spec.size(), LFG_F64, LFG_ESTIMATE, &h) == LFG_OK;
    if (h) lfg_destroy(h);
    std::printf("%s\n", ok ? "#t" : "#f");
    return 0;
  }
  if (mode == "speed") return speed(R, tmin);
  return verify(R, rounds);
}
