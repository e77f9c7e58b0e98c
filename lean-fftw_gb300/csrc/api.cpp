// C ABI of the GB300 execute path (include/lfg.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <exception>
#include <map>
#include <new>
#include <string>

#include "../../include/lfg.h"
#include "kernels.h"
#include "plan.h"
#include "ragged.h"
#include "trig.h"
#include "tuner.h"

#include "handles.h"

namespace {

thread_local std::string g_last_error;

lfg_status fail(lfg_status s, const std::string& msg) {
  g_last_error = msg;
  return s;
}

lfg_status cuda_fail(cudaError_t e, const char* what) {
  return fail(LFG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

bool smooth13(int64_t n) {
  if (n < 1) return false;
  for (int p : {2, 3, 5, 7, 11, 13})
    while (n % p == 0) n /= p;
  return n == 1;
}

int64_t tile_target() {
  const char* s = std::getenv("LFG_TILE_TARGET");
  if (s) {
    long v = std::strtol(s, nullptr, 10);
    if (v >= 16 && v <= 65536) return v;
  }
  return 2048;
}

int64_t single_max_default() {
  const char* s = std::getenv("LFG_SINGLE_MAX");
  if (s) {
    long v = std::strtol(s, nullptr, 10);
    if (v >= 2) return v;
  }
  return 2048;
}

// The kernels move whole complex elements (binary64: 16 bytes, binary32: 8 bytes), real
// lines included (read as pairs), so buffers must start on that boundary.
bool element_aligned(const void* p, int precision) {
  return ((uintptr_t)p & (precision == 0 ? 15u : 7u)) == 0;
}

// Device address of pinned (page-locked) host memory covering [p, p + bytes), or nullptr.
// On GB300 the GPU reads and writes such memory over NVLink-C2C directly, so the host entry
// points can stream the data through the kernels instead of copying it in and out first.
void* mapped_device_ptr(const void* p, size_t bytes) {
  if (!p || bytes == 0) return nullptr;
  cudaPointerAttributes a, b;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  const char* last = static_cast<const char*>(p) + bytes - 1;
  if (cudaPointerGetAttributes(&b, last) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (a.type != cudaMemoryTypeHost || b.type != cudaMemoryTypeHost || !a.devicePointer ||
      !b.devicePointer)
    return nullptr;
  if (static_cast<const char*>(b.devicePointer) - static_cast<const char*>(a.devicePointer) !=
      (ptrdiff_t)(bytes - 1))
    return nullptr;
  return a.devicePointer;
}

// Spanned scalars of a side: from the execution pointer to one past the last element.
int64_t span_scalars(const lfg::Side& s, int64_t n, int64_t howmany, int64_t per_elem) {
  return (s.offset + (n - 1) * s.stride + (howmany - 1) * s.dist + 1) * per_elem;
}

lfg_status build_chirp_device(lfg::Plan& p);

// Prime factors of n in ascending order, with multiplicity (lean-fftw `primeFactors`).
std::vector<int> prime_factors(int64_t n) {
  std::vector<int> fs;
  for (int64_t d = 2; n > 1;) {
    if (d * d > n) {
      fs.push_back((int)n);
      break;
    }
    if (n % d == 0) {
      fs.push_back((int)d);
      n /= d;
    } else {
      ++d;
    }
  }
  return fs;
}

// Small sizes with a prime factor above 13: the generic engine's own transform (generic.cu),
// the reference's operations exactly, while its direct sums stay cheap (largest factor
// <= 1024); larger ones go through Bluestein's identity, which is also more accurate there.
lfg_status build_generic_device(lfg::Plan& p) {
  const std::vector<int> fs = prime_factors(p.n);
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  p.device = dev;
  p.generic = true;
  p.ngroups = 0;
  if (p.empty) return LFG_OK;
  if ((e = lfg::prepare_generic_kernels()) != cudaSuccess) return cuda_fail(e, "kernel set-up");
  lfg::GenericDesc& g = p.gen;
  g.n = (int)p.n;
  g.nf = (int)fs.size();
  int64_t acc = 1;
  for (int i = g.nf - 1; i >= 0; --i) {
    g.f[i] = fs[i];
    acc *= fs[i];
    g.ni[i] = (int)acc;
  }
  g.lines = std::max<int64_t>(1, p.howmany) * std::max<int64_t>(1, p.howmany2);
  g.nl1 = std::max<int64_t>(1, p.howmany);
  g.in_stride = p.in.stride;
  g.in_dist = p.in.dist;
  g.in_dist2 = p.in_dist2;
  g.out_stride = p.out.stride;
  g.out_dist = p.out.dist;
  g.out_dist2 = p.out_dist2;
  g.scale = 1.0;
  const std::vector<double> tab = lfg::cos_sin_2pi_table((uint64_t)p.n);
  const size_t es = p.precision == 0 ? sizeof(double) : sizeof(float);
  e = cudaMalloc(&p.d_gen_tab, tab.size() * es);
  if (e == cudaSuccess) {
    if (p.precision == 0) {
      e = cudaMemcpy(p.d_gen_tab, tab.data(), tab.size() * es, cudaMemcpyHostToDevice);
    } else {
      std::vector<float> f(tab.begin(), tab.end());
      e = cudaMemcpy(p.d_gen_tab, f.data(), f.size() * es, cudaMemcpyHostToDevice);
    }
  }
  if (e != cudaSuccess) return cuda_fail(e, "generic twiddle table");
  g.tab = p.d_gen_tab;
  double sum = 0;
  for (int f : fs) sum += f;
  p.flops = 8.0 * (double)p.n * sum * (double)g.lines;
  return LFG_OK;
}

// Device part of a 1-D complex plan: kernels set up, autotuning, groups and tables.
lfg_status build_c2c_device(lfg::Plan& p) {
  if (!smooth13(p.n)) {
    // binary64: the reference's own algorithm where its direct sums stay cheap; binary32 (no
    // bit pattern to reproduce): Bluestein, whose error does not grow with the prime factors
    const std::vector<int> fs = prime_factors(p.n);
    if (p.precision == 0 && p.n <= lfg::kGenericMaxN && fs.back() <= 1024)
      return build_generic_device(p);
    return build_chirp_device(p);
  }
  // binary64 is bound by the FP64 pipe: two groups of small tiles (more CTAs per SM) beat one
  // group with a CTA-sized tile above 2048 points; binary32 is bound by HBM: as few groups as fit.
  // A lone contiguous binary64 transform of up to kClusterMaxN points stays one group, which
  // the thread-block cluster kernel runs.
  if (p.single_max == 0 && p.precision == 0 && p.howmany == 1 && p.howmany2 == 1 &&
      p.n <= lfg::kClusterMaxN && p.in.stride == 1 && p.out.stride == 1)
    p.single_max = lfg::kClusterMaxN;
  if (p.single_max == 0 && p.precision == 0) p.single_max = single_max_default();
  if (p.single_max == 0 && p.precision == 1) p.single_max = lfg::kF32SingleGroupMax;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  p.device = dev;
  if (!p.empty) {
    e = p.precision == 0 ? lfg::prepare_group_kernels_f64() : lfg::prepare_group_kernels_f32();
    if (e != cudaSuccess) return cuda_fail(e, "kernel set-up");
    if (p.measure && p.howmany2 == 1) {
      std::string msg = lfg::tune_c2c(p, tile_target());
      if (!msg.empty()) return fail(LFG_ERR_CUDA, msg);
    }
    std::string msg = lfg::build_c2c(p, p.tile > 0 ? p.tile : tile_target());
    if (!msg.empty()) {
      lfg::free_plan_memory(p);
      return fail(LFG_ERR_UNSUPPORTED, msg);
    }
  }
  return LFG_OK;
}

// Smallest 13-smooth integer >= m.
int64_t next_smooth(int64_t m) {
  while (!smooth13(m)) ++m;
  return m;
}

// Bluestein plan for a size with a prime factor above 13 (chirp.cu explains the identity):
// chirp table, the filter's spectrum (computed once, in binary64, by a transform of length
// L), and forward/backward transforms of length L over all lines of the batch.
lfg_status build_chirp_device(lfg::Plan& p) {
  const int64_t n = p.n;
  if (n < 2 || n > ((int64_t)1 << 24)) return fail(LFG_ERR_UNSUPPORTED, "size outside 2..2^24");
  const int64_t L = next_smooth(2 * n - 1);
  const int64_t lines = std::max<int64_t>(1, p.howmany) * std::max<int64_t>(1, p.howmany2);
  if (lines * L >= ((int64_t)1 << 31))
    return fail(LFG_ERR_UNSUPPORTED, "batch too large for the chirp-z path (2^31 elements)");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  p.device = dev;
  p.ngroups = 0;
  if (p.empty) return LFG_OK;
  // chirp c_m = exp(s pi i m^2 / n) = cos/sin(2 pi t / 2n), t = m^2 mod 2n (exact table)
  const std::vector<double> tab = lfg::cos_sin_2pi_table((uint64_t)(2 * n));
  const double sg = p.fwd ? -1.0 : 1.0;
  std::vector<double> c(2 * n), b(2 * L, 0.0);
  for (int64_t m = 0; m < n; ++m) {
    const int64_t t = (m * m) % (2 * n);   // m < 2^24: no overflow
    c[2 * m] = tab[2 * t];
    c[2 * m + 1] = sg * tab[2 * t + 1];
    // the filter conj(c_m) at m and at L - m
    b[2 * m] = c[2 * m];
    b[2 * m + 1] = -c[2 * m + 1];
    if (m > 0) {
      b[2 * (L - m)] = c[2 * m];
      b[2 * (L - m) + 1] = -c[2 * m + 1];
    }
  }
  // its forward transform in binary64
  std::vector<double> bh(2 * L);
  {
    lfg::Plan t;
    t.kind = lfg::Kind::C2C;
    t.precision = 0;
    t.fwd = true;
    t.n = L;
    t.howmany = 1;
    t.in = t.out = {0, 1, L};
    t.radices = lfg::choose_radices(L, 0);
    lfg_status s = build_c2c_device(t);
    if (s != LFG_OK) return s;
    void* db = nullptr;
    e = cudaMalloc(&db, 2 * 2 * L * sizeof(double));
    if (e == cudaSuccess) e = cudaMemcpy(db, b.data(), 2 * L * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
      e = lfg::execute_plan(t, db, static_cast<double*>(db) + 2 * L, nullptr);
    if (e == cudaSuccess)
      e = cudaMemcpy(bh.data(), static_cast<double*>(db) + 2 * L, 2 * L * sizeof(double),
                     cudaMemcpyDeviceToHost);
    if (db) cudaFree(db);
    lfg::free_plan_memory(t);
    if (e != cudaSuccess) return cuda_fail(e, "chirp filter transform");
  }
  // chirp and filter spectrum on the device, in the plan's precision
  const size_t es = p.precision == 0 ? sizeof(double) : sizeof(float);
  e = cudaMalloc(&p.d_chirp_tab, 2 * (size_t)(n + L) * es);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc of the chirp tables");
  std::vector<double> both(c);
  both.insert(both.end(), bh.begin(), bh.end());
  if (p.precision == 0) {
    e = cudaMemcpy(p.d_chirp_tab, both.data(), both.size() * es, cudaMemcpyHostToDevice);
  } else {
    std::vector<float> f(both.begin(), both.end());
    e = cudaMemcpy(p.d_chirp_tab, f.data(), f.size() * es, cudaMemcpyHostToDevice);
  }
  if (e != cudaSuccess) return cuda_fail(e, "chirp table upload");
  // forward and backward transforms of length L over all lines (dense, out of place)
  for (int dir = 0; dir < 2; ++dir) {
    auto q = std::make_shared<lfg::Plan>();
    q->kind = lfg::Kind::C2C;
    q->precision = p.precision;
    q->fwd = dir == 0;
    q->n = L;
    q->howmany = lines;
    q->in = q->out = {0, 1, L};
    q->no_comp = p.no_comp;
    q->radices = lfg::choose_radices(L, p.precision);
    lfg_status s = build_c2c_device(*q);
    if (s != LFG_OK) return s;
    if (dir == 1 && q->ngroups >= 1) q->groups[q->ngroups - 1].scale = 1.0 / (double)L;
    (dir == 0 ? p.chirp_fwd : p.chirp_bwd) = q;
  }
  const size_t ces = p.precision == 0 ? 16 : 8;
  e = cudaMalloc(&p.d_chirp_buf, 2 * (size_t)lines * (size_t)L * ces);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc of the chirp buffers");
  lfg::ChirpDesc& d = p.chirp;
  d.n = n;
  d.L = L;
  d.lines = lines;
  d.nl1 = std::max<int64_t>(1, p.howmany);
  d.in_off = d.out_off = 0;
  d.in_stride = p.in.stride;
  d.in_dist = p.in.dist;
  d.in_dist2 = p.in_dist2;
  d.out_stride = p.out.stride;
  d.out_dist = p.out.dist;
  d.out_dist2 = p.out_dist2;
  d.fd_L = lfg::make_fastdiv((int)L);
  d.fd_n = lfg::make_fastdiv((int)n);
  d.fd_nl1 = lfg::make_fastdiv((int)d.nl1);
  d.chirp = p.d_chirp_tab;
  d.bhat = static_cast<const char*>(p.d_chirp_tab) + 2 * (size_t)n * es;
  p.radices = p.chirp_fwd->radices;
  p.flops = 2 * p.chirp_fwd->flops + 18.0 * (double)(lines * L);
  return LFG_OK;
}

lfg_status finish_c2c(lfg::Plan& p, lfg_plan** out) {
  lfg_status s = build_c2c_device(p);
  if (s != LFG_OK) return s;
  p.in_span = span_scalars(p.in, p.n, p.howmany, 2);
  p.out_span = span_scalars(p.out, p.n, p.howmany, 2);
  lfg_plan* h = new (std::nothrow) lfg_plan;
  if (!h) {
    lfg::free_plan_memory(p);
    return fail(LFG_ERR_NOMEM, "host allocation");
  }
  h->p = p;
  *out = h;
  return LFG_OK;
}

lfg_status finish_real(lfg::Plan& p, const lfg::RealLayout& L, lfg_plan** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  p.device = dev;
  p.howmany = L.howmany;
  p.n = L.n;
  const int64_t M = L.n / 2;
  // spans: real side in doubles, complex side in doubles (2 per element)
  const int64_t rspan = L.r_off + (L.howmany - 1) * L.r_bdist + (L.n0 - 1) * L.r_rdist + L.n;
  const int64_t cspan = 2 * (L.c_off + (L.howmany - 1) * L.c_bdist + (L.n0 - 1) * L.c_rdist + M + 1);
  const bool r2c = p.kind == lfg::Kind::R2C;
  p.in_span = r2c ? rspan : cspan;
  p.out_span = r2c ? cspan : rspan;
  if (!p.empty) {
    // the column pass of a rank-2 plan runs the group kernels of the plan's precision
    e = p.precision == 0 ? lfg::prepare_group_kernels_f64() : lfg::prepare_group_kernels_f32();
    if (e != cudaSuccess) return cuda_fail(e, "kernel set-up");
    if ((e = lfg::prepare_real_kernels()) != cudaSuccess) return cuda_fail(e, "kernel set-up");
    std::string msg = lfg::build_real(p, L, tile_target());
    if (!msg.empty()) {
      lfg::free_plan_memory(p);
      return fail(LFG_ERR_UNSUPPORTED, msg);
    }
  }
  lfg_plan* h = new (std::nothrow) lfg_plan;
  if (!h) {
    lfg::free_plan_memory(p);
    return fail(LFG_ERR_NOMEM, "host allocation");
  }
  h->p = p;
  *out = h;
  return LFG_OK;
}

lfg_status plan_real_common(bool r2c, size_t n0, size_t n, size_t howmany, lfg_precision precision,
                            unsigned flags, lfg_plan** out) {
  if (!out) return fail(LFG_ERR_INVALID, "null output handle");
  *out = nullptr;
  if (precision != LFG_F64 && precision != LFG_F32) return fail(LFG_ERR_INVALID, "bad precision");
  if (n < 2 || n0 < 1) return fail(LFG_ERR_UNSUPPORTED, "sizes must be >= 2 (last) and >= 1");
  if (n & 1) return fail(LFG_ERR_UNSUPPORTED, "odd-length real transforms are not executed");
  if (!smooth13((int64_t)n) || !smooth13((int64_t)n0))
    return fail(LFG_ERR_UNSUPPORTED, "sizes must be 13-smooth");
  lfg::Plan p;
  p.kind = r2c ? lfg::Kind::R2C : lfg::Kind::C2R;
  p.precision = precision;
  p.fwd = r2c;
  p.empty = howmany == 0;
  lfg::RealLayout L;
  L.n0 = (int64_t)n0;
  L.n = (int64_t)n;
  L.howmany = std::max<int64_t>(1, (int64_t)howmany);
  L.r_rdist = (int64_t)n;
  L.r_bdist = (int64_t)(n0 * n);
  L.c_rdist = (int64_t)(n / 2 + 1);
  L.c_bdist = (int64_t)(n0 * (n / 2 + 1));
  if ((flags & LFG_ADJOINT) && n0 > 1) return fail(LFG_ERR_UNSUPPORTED, "adjoint scaling is 1-D only");
  p.real.adjoint = (flags & LFG_ADJOINT) ? 1 : 0;
  p.generic_kernels = (flags & LFG_GENERIC_KERNELS) != 0;
  return finish_real(p, L, out);
}

lfg_status plan_1d_common(size_t n, int sign, size_t howmany, lfg_precision precision,
                          const int* radices, int npass, lfg_plan** out, unsigned flags = 0) {
  if (!out) return fail(LFG_ERR_INVALID, "null output handle");
  *out = nullptr;
  if (sign != -1 && sign != 1) return fail(LFG_ERR_INVALID, "sign must be -1 or +1");
  if (precision != LFG_F64 && precision != LFG_F32) return fail(LFG_ERR_INVALID, "bad precision");
  if (n < 2 || n > ((size_t)1 << 24)) return fail(LFG_ERR_UNSUPPORTED, "size outside 2..2^24");
  if (radices && !smooth13((int64_t)n))
    return fail(LFG_ERR_UNSUPPORTED, "explicit radix sequences need a 13-smooth size");
  lfg::Plan p;
  p.kind = lfg::Kind::C2C;
  p.precision = precision;
  p.fwd = sign < 0;
  p.n = (int64_t)n;
  p.howmany = (int64_t)howmany;
  p.in.stride = p.out.stride = 1;
  p.in.dist = p.out.dist = (int64_t)n;
  p.empty = howmany == 0;
  p.no_comp = (flags & LFG_NO_COMPENSATION) != 0;
  p.wait_give_up = (flags & LFG_TEST_WAIT_GIVE_UP) != 0;
  p.generic_kernels = (flags & LFG_GENERIC_KERNELS) != 0;
  p.measure = (flags & LFG_MEASURE) != 0 && !radices;
  if (radices) {
    if (npass < 1 || npass > lfg::kMaxPass) return fail(LFG_ERR_INVALID, "bad pass count");
    p.radices.assign(radices, radices + npass);
    p.radices_given = true;
  } else if (howmany == 1 && precision == LFG_F64 && p.n <= lfg::kClusterMaxN && !p.measure) {
    // a lone transform runs on a thread-block cluster: the radices of least latency
    p.radices = lfg::choose_radices_latency(p.n);
  } else {
    p.radices = lfg::choose_radices(p.n, precision);
  }
  return finish_c2c(p, out);
}

// A dimension of the FFI spec in complex elements.
struct CDim {
  int64_t n, is, os;
};

// One r2r axis stage: lines of n real elements (`is`/`os` apart) in a batch of inner x outer
// lines; the embedding of each line goes through a complex DFT of the embedding size.
lfg_status build_r2r_child(lfg::Plan& c, int rkind, int64_t n, int64_t is, int64_t os,
                           const CDim& inner, const CDim& outer, lfg_precision precision,
                           unsigned flags) {
  const int64_t M = lfg::r2r_embed_size(rkind, n);
  if (M == 0) return fail(LFG_ERR_UNSUPPORTED, "r2r kind or size not defined (REDFT00 needs n >= 2)");
  if (M > ((int64_t)1 << 24))
    return fail(LFG_ERR_UNSUPPORTED, "r2r embedding size " + std::to_string(M) + " above 2^24");
  const int64_t lines = inner.n * outer.n;
  if (lines * M >= ((int64_t)1 << 31) || lines * n >= ((int64_t)1 << 31))
    return fail(LFG_ERR_UNSUPPORTED, "r2r batch too large (2^31 embedded elements per plan)");
  c.kind = lfg::Kind::R2R;
  c.precision = precision;
  c.fwd = rkind != lfg::kHC2R;
  c.n = n;
  c.howmany = lines;
  lfg::R2RDesc& d = c.r2r;
  d.kind = rkind;
  d.n = n;
  d.M = M;
  d.lines = lines;
  d.nl1 = std::max<int64_t>(1, inner.n);
  d.in_off = d.out_off = 0;
  d.in_stride = is;
  d.out_stride = os;
  d.in_dist = inner.is;
  d.out_dist = inner.os;
  d.in_dist2 = outer.is;
  d.out_dist2 = outer.os;
  d.fd_m = lfg::make_fastdiv((int)M);
  d.fd_n = lfg::make_fastdiv((int)n);
  d.fd_nl1 = lfg::make_fastdiv((int)d.nl1);
  int dev = 0;
  cudaGetDevice(&dev);
  c.device = dev;
  const size_t ces = precision == 0 ? 16 : 8;
  cudaError_t e = cudaMalloc(&c.d_r2r_buf, 2 * (size_t)lines * (size_t)M * ces);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc of the r2r buffers");
  if (M > 1) {
    auto dft = std::make_shared<lfg::Plan>();
    dft->kind = lfg::Kind::C2C;
    dft->precision = precision;
    dft->fwd = c.fwd;
    dft->n = M;
    dft->howmany = lines;
    dft->in = dft->out = {0, 1, M};
    dft->no_comp = (flags & LFG_NO_COMPENSATION) != 0;
    dft->radices = lfg::choose_radices(M, precision);
    lfg_status s = build_c2c_device(*dft);
    if (s != LFG_OK) return s;
    c.flops = dft->flops;
    c.r2r_dft = dft;
  }
  return LFG_OK;
}

// Multi-axis transforms, separable along each axis (lean-fftw's generic engine applies a
// line operation along each axis over all other indices: `alongAxis`,
// LeanFFTW/Core/Problem.lean:170-212).  Complex problems (rank >= 2, or vector rank >= 2) and
// all r2r problems become one stage per axis, last axis first (complex axes of size 1 are
// skipped), each an ordinary 1-D plan whose batch is every other dimension: dimensions that
// nest (outer stride = inner count x inner stride on both sides) are merged, the two
// innermost remaining ones are covered by one launch (lines, and blocks of lines), any
// further ones by a host loop of launches.  The first stage reads the input; the later
// stages work in place on the output.  Units: complex elements (c2c) or real scalars (r2r).
lfg_status build_separable(lfg::Plan& p, bool r2r, const std::vector<CDim>& T,
                           const std::vector<CDim>& V, const std::vector<int>& kinds,
                           int64_t in_off, int64_t out_off, int sign, lfg_precision precision,
                           unsigned flags) {
  p.kind = r2r ? lfg::Kind::R2R : lfg::Kind::C2C;
  p.precision = precision;
  p.fwd = sign < 0;
  p.n = 1;
  p.howmany = 1;
  for (const CDim& d : T) p.n *= d.n;
  for (const CDim& d : V) p.howmany *= d.n;
  p.empty = p.howmany == 0;
  p.in.offset = in_off;
  p.out.offset = out_off;
  int64_t ihi = in_off, ohi = out_off;
  for (const auto* L : {&T, &V})
    for (const CDim& d : *L)
      if (d.n > 1) {
        ihi += (d.n - 1) * d.is;
        ohi += (d.n - 1) * d.os;
      }
  int dev = 0;
  cudaGetDevice(&dev);
  p.device = dev;
  if (!p.empty) {
    std::vector<int> axes;
    for (int d = (int)T.size() - 1; d >= 0; --d)
      if (T[d].n > 1 || r2r) axes.push_back(d);
    if (axes.empty()) return fail(LFG_ERR_UNSUPPORTED, "all transform dimensions are 1 (a copy)");
    for (size_t k = 0; k < axes.size(); ++k) {
      const int d = axes[k];
      const bool first = k == 0;
      auto is_of = [&](const CDim& x) { return first ? x.is : x.os; };
      std::vector<CDim> batch;
      for (int e = 0; e < (int)T.size(); ++e)
        if (e != d && T[e].n > 1) batch.push_back({T[e].n, is_of(T[e]), T[e].os});
      for (const CDim& v : V)
        if (v.n > 1) batch.push_back({v.n, is_of(v), v.os});
      std::sort(batch.begin(), batch.end(), [](const CDim& a, const CDim& b) {
        return a.os != b.os ? a.os < b.os : a.is < b.is;
      });
      for (size_t i = 0; i + 1 < batch.size();) {
        CDim& a = batch[i];
        const CDim& b = batch[i + 1];
        if (b.is == a.n * a.is && b.os == a.n * a.os) {
          a.n *= b.n;
          batch.erase(batch.begin() + i + 1);
        } else {
          ++i;
        }
      }
      const CDim inner = batch.size() > 0 ? batch[0] : CDim{1, 0, 0};
      const CDim outer = batch.size() > 1 ? batch[1] : CDim{1, 0, 0};
      lfg::AxisStage stage;
      int64_t nl = 1;
      for (size_t i = 2; i < batch.size(); ++i) nl *= batch[i].n;
      if (nl > (1 << 16)) {
        lfg::free_plan_memory(p);
        return fail(LFG_ERR_UNSUPPORTED, "too many launches for this dimension nesting");
      }
      for (int64_t q = 0; q < nl; ++q) {
        int64_t r = q, oi = first ? in_off : out_off, oo = out_off;
        for (size_t i = 2; i < batch.size(); ++i) {
          oi += (r % batch[i].n) * batch[i].is;
          oo += (r % batch[i].n) * batch[i].os;
          r /= batch[i].n;
        }
        stage.loops.push_back({oi, oo});
      }
      auto st = std::make_shared<lfg::Plan>();
      lfg::Plan& c = *st;
      lfg_status s;
      if (r2r) {
        s = build_r2r_child(c, kinds[d], T[d].n, is_of(T[d]), T[d].os, inner, outer, precision, flags);
      } else {
        c.kind = lfg::Kind::C2C;
        c.precision = precision;
        c.fwd = p.fwd;
        c.n = T[d].n;
        c.in = {0, is_of(T[d]), inner.is};
        c.out = {0, T[d].os, inner.os};
        c.howmany = inner.n;
        c.howmany2 = outer.n;
        c.in_dist2 = outer.is;
        c.out_dist2 = outer.os;
        c.no_comp = (flags & LFG_NO_COMPENSATION) != 0;
        c.radices = lfg::choose_radices(c.n, precision);
        s = build_c2c_device(c);
      }
      if (s != LFG_OK) {
        lfg::free_plan_memory(c);
        lfg::free_plan_memory(p);
        return s;
      }
      p.flops += c.flops * (double)nl;
      const std::vector<int>& rs = r2r && c.r2r_dft ? c.r2r_dft->radices : c.radices;
      p.radices.insert(p.radices.end(), rs.begin(), rs.end());
      stage.plan = st;
      p.stages.push_back(std::move(stage));
    }
  }
  const int64_t per = r2r ? 1 : 2;
  p.in_span = per * (ihi + 1);
  p.out_span = per * (ohi + 1);
  return LFG_OK;
}

lfg_status wrap_plan(lfg::Plan& p, lfg_plan** out) {
  lfg_plan* h = new (std::nothrow) lfg_plan;
  if (!h) {
    lfg::free_plan_memory(p);
    return fail(LFG_ERR_NOMEM, "host allocation");
  }
  h->p = p;
  *out = h;
  return LFG_OK;
}

lfg_status plan_separable(bool r2r, const std::vector<CDim>& T, const std::vector<CDim>& V,
                          const std::vector<int>& kinds, int64_t in_off, int64_t out_off,
                          int sign, lfg_precision precision, unsigned flags, lfg_plan** out) {
  lfg::Plan p;
  lfg_status s = build_separable(p, r2r, T, V, kinds, in_off, out_off, sign, precision, flags);
  if (s != LFG_OK) return s;
  return wrap_plan(p, out);
}

// ---- problems through dense buffers (gather, inner plans, scatter) --------------------------

// Dense row-major complex dimensions (complex units) of extents ns, as CDims.
std::vector<CDim> dense_dims(const std::vector<int64_t>& ns) {
  std::vector<CDim> d(ns.size());
  int64_t acc = 1;
  for (int k = (int)ns.size() - 1; k >= 0; --k) {
    d[k] = CDim{ns[k], acc, acc};
    acc *= ns[k];
  }
  return d;
}

lfg::PackDesc pack_desc(int mode, const std::vector<int64_t>& ns, const std::vector<int64_t>& st,
                        int64_t re_off, int64_t im_off, int64_t half, int64_t total) {
  lfg::PackDesc d{};
  d.ndims = (int)ns.size();
  d.mode = mode;
  for (size_t k = 0; k < ns.size(); ++k) {
    d.n[k] = ns[k];
    d.st[k] = st[k];
  }
  d.re_off = re_off;
  d.im_off = im_off;
  d.half = half;
  d.total = total;
  return d;
}

// Highest scalar offset reached from base `off` over extents ns with strides st; -1 if some
// offset would be negative.
int64_t reach(int64_t off, const std::vector<int64_t>& ns, const std::vector<int64_t>& st) {
  int64_t lo = off, hi = off;
  for (size_t k = 0; k < ns.size(); ++k)
    if (ns[k] > 1) {
      const int64_t e = (ns[k] - 1) * st[k];
      (e > 0 ? hi : lo) += e;
    }
  return lo < 0 ? -1 : hi;
}

// A dimension of the FFI spec in real scalars (any sign of stride).
struct SDim {
  int64_t n, is, os;
};

// Complex DFT of any layout: gather to dense, transform there, scatter.
lfg_status plan_c2c_packed(const std::vector<SDim>& T, const std::vector<SDim>& V, int64_t inRe,
                           int64_t inIm, int64_t outRe, int64_t outIm, int sign,
                           lfg_precision precision, unsigned flags, lfg_plan** out) {
  std::vector<int64_t> ns, is, os;
  for (const SDim& d : V) ns.push_back(d.n), is.push_back(d.is), os.push_back(d.os);
  for (const SDim& d : T) ns.push_back(d.n), is.push_back(d.is), os.push_back(d.os);
  if ((int)ns.size() > lfg::kPackMaxDims) return fail(LFG_ERR_UNSUPPORTED, "more than 8 dimensions");
  int64_t total = 1;
  for (int64_t n : ns) total *= n;
  lfg::Plan p;
  p.kind = lfg::Kind::C2C;
  p.precision = precision;
  p.fwd = sign < 0;
  p.empty = total == 0;
  p.n = 1;
  for (const SDim& d : T) p.n *= d.n;
  p.howmany = p.n > 0 ? total / std::max<int64_t>(1, p.n) : 0;
  const int64_t ih = std::max(reach(inRe, ns, is), reach(inIm, ns, is));
  const int64_t oh = std::max(reach(outRe, ns, os), reach(outIm, ns, os));
  if (reach(inRe, ns, is) < 0 || reach(inIm, ns, is) < 0 || reach(outRe, ns, os) < 0 ||
      reach(outIm, ns, os) < 0)
    return fail(LFG_ERR_UNSUPPORTED, "strides reach below the buffer start");
  p.in_span = ih + 1;
  p.out_span = oh + 1;
  int dev = 0;
  cudaGetDevice(&dev);
  p.device = dev;
  if (!p.empty) {
    std::vector<int64_t> tn;
    for (const SDim& d : T) tn.push_back(d.n);
    const std::vector<CDim> dd = dense_dims(ns);
    std::vector<CDim> Vd(dd.begin(), dd.begin() + V.size()), Td(dd.begin() + V.size(), dd.end());
    auto inner = std::make_shared<lfg::Plan>();
    lfg_status s = build_separable(*inner, false, Td, Vd, {}, 0, 0, sign, precision, flags);
    if (s != LFG_OK) return s;
    p.pack_elems = total;
    const size_t ces = precision == 0 ? 16 : 8;
    if (cudaMalloc(&p.d_pack_buf, 2 * (size_t)total * ces) != cudaSuccess) {
      lfg::free_plan_memory(*inner);
      return fail(LFG_ERR_NOMEM, "cudaMalloc of the dense buffers");
    }
    p.steps.push_back({lfg::PackStep::kGather,
                       pack_desc(lfg::kPackComplex, ns, is, inRe, inIm, 0, total), nullptr, 0, 2});
    p.steps.push_back({lfg::PackStep::kPlan, {}, inner, 2, 3});
    p.steps.push_back({lfg::PackStep::kScatter,
                       pack_desc(lfg::kPackComplex, ns, os, outRe, outIm, 0, total), nullptr, 3, 1});
    p.flops = inner->flops;
    p.radices = inner->radices;
  }
  return wrap_plan(p, out);
}

// rdft2 of any layout (rank >= 1; odd, non-smooth or strided sizes; split complex side), as the
// generic engine computes it (Core/Problem.lean:142-150, 222-236): r2c = the complex forward
// transform of the real data (imaginary parts 0) over every axis, first n/2+1 values of the
// last; c2r = complex backward transforms along the other axes of the half spectrum, then the
// Hermitian extension along the last axis, its backward transform, real parts.
lfg_status plan_rdft2_packed(bool r2c, const std::vector<SDim>& T, const std::vector<SDim>& V,
                             int64_t rRe, int64_t cRe, int64_t cIm, lfg_precision precision,
                             unsigned flags, lfg_plan** out) {
  const int r = (int)T.size();
  std::vector<int64_t> ns, rst, cst;   // full extents; real-side and complex-side strides
  for (const SDim& d : V) {
    ns.push_back(d.n);
    rst.push_back(r2c ? d.is : d.os);
    cst.push_back(r2c ? d.os : d.is);
  }
  for (const SDim& d : T) {
    ns.push_back(d.n);
    rst.push_back(r2c ? d.is : d.os);
    cst.push_back(r2c ? d.os : d.is);
  }
  if ((int)ns.size() > lfg::kPackMaxDims) return fail(LFG_ERR_UNSUPPORTED, "more than 8 dimensions");
  const int64_t nl = T[r - 1].n, h = nl / 2 + 1;
  std::vector<int64_t> hs = ns;
  hs.back() = h;
  int64_t total = 1, htotal = 1;
  for (int64_t n : ns) total *= n;
  for (int64_t n : hs) htotal *= n;
  const int64_t rreach = reach(rRe, ns, rst);
  const int64_t creach = std::max(reach(cRe, hs, cst), reach(cIm, hs, cst));
  if (rreach < 0 || reach(cRe, hs, cst) < 0 || reach(cIm, hs, cst) < 0)
    return fail(LFG_ERR_UNSUPPORTED, "strides reach below the buffer start");
  lfg::Plan p;
  p.kind = r2c ? lfg::Kind::R2C : lfg::Kind::C2R;
  p.precision = precision;
  p.fwd = r2c;
  p.empty = total == 0;
  p.n = nl;
  p.in_span = (r2c ? rreach : creach) + 1;
  p.out_span = (r2c ? creach : rreach) + 1;
  int dev = 0;
  cudaGetDevice(&dev);
  p.device = dev;
  if (p.empty) return wrap_plan(p, out);
  const size_t ces = precision == 0 ? 16 : 8;
  p.pack_elems = total;
  if (cudaMalloc(&p.d_pack_buf, 2 * (size_t)total * ces) != cudaSuccess)
    return fail(LFG_ERR_NOMEM, "cudaMalloc of the dense buffers");
  const int nv = (int)V.size();
  auto fail_free = [&](lfg_status s) {
    lfg::free_plan_memory(p);
    return s;
  };
  if (r2c) {
    const std::vector<CDim> dd = dense_dims(ns);
    std::vector<CDim> Vd(dd.begin(), dd.begin() + nv), Td(dd.begin() + nv, dd.end());
    auto inner = std::make_shared<lfg::Plan>();
    lfg_status s = build_separable(*inner, false, Td, Vd, {}, 0, 0, -1, precision, flags);
    if (s != LFG_OK) return fail_free(s);
    p.steps.push_back({lfg::PackStep::kGather, pack_desc(lfg::kPackReal, ns, rst, rRe, -1, 0, total),
                       nullptr, 0, 2});
    p.steps.push_back({lfg::PackStep::kPlan, {}, inner, 2, 3});
    p.steps.push_back({lfg::PackStep::kScatter,
                       pack_desc(lfg::kPackComplex, ns, cst, cRe, cIm, h, htotal), nullptr, 3, 1});
    p.flops = inner->flops;
  } else {
    // half spectrum, dense (extents hs) in buffer 2
    p.steps.push_back({lfg::PackStep::kGather, pack_desc(lfg::kPackComplex, hs, cst, cRe, cIm, 0, htotal),
                       nullptr, 0, 2});
    bool cols = false;
    for (int k = 0; k + 1 < r; ++k) cols = cols || T[k].n > 1;
    if (cols) {
      // backward transforms along axes 0..r-2 of the half spectrum, in place
      const std::vector<CDim> dd = dense_dims(hs);
      std::vector<CDim> Vd(dd.begin(), dd.begin() + nv), Td(dd.begin() + nv, dd.end() - 1);
      Vd.push_back(dd.back());
      auto inner = std::make_shared<lfg::Plan>();
      lfg_status s = build_separable(*inner, false, Td, Vd, {}, 0, 0, 1, precision, flags);
      if (s != LFG_OK) return fail_free(s);
      p.steps.push_back({lfg::PackStep::kPlan, {}, inner, 2, 2});
      p.flops += inner->flops;
    }
    // Hermitian extension along the last axis (dense half -> dense full, buffer 3)
    std::vector<int64_t> hst(hs.size());
    {
      int64_t acc = 1;
      for (int k = (int)hs.size() - 1; k >= 0; --k) {
        hst[k] = 2 * acc;
        acc *= hs[k];
      }
    }
    p.steps.push_back({lfg::PackStep::kGather, pack_desc(lfg::kPackHerm, ns, hst, 0, 1, h, total),
                       nullptr, 2, 3});
    // backward transform of every row of the last axis, then the real parts
    auto rows = std::make_shared<lfg::Plan>();
    const std::vector<CDim> T1{{nl, 1, 1}}, V1{{total / nl, nl, nl}};
    lfg_status s = build_separable(*rows, false, T1, V1, {}, 0, 0, 1, precision, flags);
    if (s != LFG_OK) return fail_free(s);
    p.steps.push_back({lfg::PackStep::kPlan, {}, rows, 3, 2});
    p.flops += rows->flops;
    p.steps.push_back({lfg::PackStep::kScatter, pack_desc(lfg::kPackReal, ns, rst, rRe, -1, 0, total),
                       nullptr, 2, 1});
  }
  return wrap_plan(p, out);
}

using lfg::guarded;

}  // namespace

void lfg::set_last_error(const std::string& msg) { g_last_error = msg; }

extern "C" {

static lfg_status lfg_plan_1d_impl(size_t n, int sign, size_t howmany, lfg_precision precision,
                       unsigned flags, lfg_plan** out) {
  return plan_1d_common(n, sign, howmany, precision, nullptr, 0, out, flags);
}

static lfg_status lfg_plan_r2c_impl(size_t n, size_t howmany, lfg_precision precision, unsigned flags,
                        lfg_plan** out) {
  return plan_real_common(true, 1, n, howmany, precision, flags, out);
}

static lfg_status lfg_plan_c2r_impl(size_t n, size_t howmany, lfg_precision precision, unsigned flags,
                        lfg_plan** out) {
  return plan_real_common(false, 1, n, howmany, precision, flags, out);
}

static lfg_status lfg_plan_r2c_2d_impl(size_t n0, size_t n1, size_t howmany, lfg_precision precision,
                           unsigned flags, lfg_plan** out) {
  return plan_real_common(true, n0, n1, howmany, precision, flags, out);
}

static lfg_status lfg_plan_c2r_2d_impl(size_t n0, size_t n1, size_t howmany, lfg_precision precision,
                           unsigned flags, lfg_plan** out) {
  return plan_real_common(false, n0, n1, howmany, precision, flags, out);
}

static lfg_status lfg_plan_r2r_impl(size_t n, int kind, size_t howmany, lfg_precision precision,
                        unsigned flags, lfg_plan** out) {
  if (!out) return fail(LFG_ERR_INVALID, "null output handle");
  *out = nullptr;
  if (precision != LFG_F64 && precision != LFG_F32) return fail(LFG_ERR_INVALID, "bad precision");
  if (kind < 0 || kind > 10) return fail(LFG_ERR_INVALID, "r2r kind outside 0..10");
  if (n < 1) return fail(LFG_ERR_INVALID, "size must be >= 1");
  const std::vector<CDim> T{{(int64_t)n, 1, 1}}, V{{(int64_t)howmany, (int64_t)n, (int64_t)n}};
  return plan_separable(true, T, V, {kind}, 0, 0, -1, precision, flags, out);
}

static lfg_status lfg_plan_1d_radices_impl(size_t n, int sign, size_t howmany, lfg_precision precision,
                               const int* radices, int npass, lfg_plan** out) {
  if (!radices) return fail(LFG_ERR_INVALID, "null radices");
  return plan_1d_common(n, sign, howmany, precision, radices, npass, out);
}

// Decode lean-fftw's problem encoding (LeanFFTW/FFI.lean:32-47) and plan the parts this
// library executes.  Strides and offsets arrive in doubles.
static lfg_status lfg_plan_spec_impl(const double* spec, size_t nspec, lfg_precision precision,
                         unsigned flags, lfg_plan** out) {
  if (!out) return fail(LFG_ERR_INVALID, "null output handle");
  *out = nullptr;
  if (!spec || nspec < 8) return fail(LFG_ERR_INVALID, "spec too short");
  for (size_t i = 0; i < nspec; ++i)
    if (!std::isfinite(spec[i]) || spec[i] != std::floor(spec[i]))
      return fail(LFG_ERR_INVALID, "spec entries must be integers");
  const int kind = (int)spec[0];
  const int sign = spec[1] < 0 ? -1 : 1;
  const int64_t rank = (int64_t)spec[2], vrank = (int64_t)spec[3];
  if (rank < 0 || vrank < 0 || nspec < (size_t)(8 + 3 * (rank + vrank)))
    return fail(LFG_ERR_INVALID, "spec length does not match rank and vector rank");
  const int64_t inRe = (int64_t)spec[4], inIm = (int64_t)spec[5];
  const int64_t outRe = (int64_t)spec[6], outIm = (int64_t)spec[7];
  auto dim = [&](int64_t i, int64_t* n, int64_t* is, int64_t* os) {
    *n = (int64_t)spec[8 + 3 * i];
    *is = (int64_t)spec[9 + 3 * i];
    *os = (int64_t)spec[10 + 3 * i];
  };
  // offsets and strides count real scalars of the plan's precision (doubles or floats)
  if (precision != LFG_F64 && precision != LFG_F32) return fail(LFG_ERR_INVALID, "bad precision");
  // all dimensions, in real scalars (any sign of stride)
  std::vector<SDim> ST, SV;
  for (int64_t i = 0; i < rank + vrank; ++i) {
    int64_t n, is, os;
    dim(i, &n, &is, &os);
    if (n < 0) return fail(LFG_ERR_INVALID, "negative dimension");
    if (i < rank && n < 1) return fail(LFG_ERR_UNSUPPORTED, "transform dimension must be >= 1");
    if (i < rank && n > ((int64_t)1 << 24)) return fail(LFG_ERR_UNSUPPORTED, "transform sizes above 2^24");
    (i < rank ? ST : SV).push_back(SDim{n, is, os});
  }
  if (kind == 1) {
    // rdft2 (Core/Problem.lean:222-236): r2c when sign < 0 (real input), else c2r; the last
    // dimension is halved on the complex side.  The fused kernels take rank 1 or 2, vector
    // rank <= 1, unit stride along the last axis on both sides, an interleaved complex side and
    // an even 13-smooth size; everything else goes through dense buffers and complex transforms.
    if (rank < 1) return fail(LFG_ERR_UNSUPPORTED, "rdft2 needs rank >= 1");
    const bool r2c = sign < 0;
    const int64_t rRe = r2c ? inRe : outRe;
    const int64_t cRe = r2c ? outRe : inRe, cIm = r2c ? outIm : inIm;
    const SDim last = ST[rank - 1];
    const int64_t rstl = r2c ? last.is : last.os, cstl = r2c ? last.os : last.is;
    bool native = rank <= 2 && vrank <= 1 && cIm == cRe + 1 && !(cRe & 1) && rRe >= 0 && cRe >= 0 &&
                  (rRe & 1) == 0 && rstl == 1 && cstl == 2 && last.n >= 2 && !(last.n & 1) &&
                  smooth13(last.n) && (rank == 1 || smooth13(ST[0].n));
    lfg::RealLayout L;
    L.n = last.n;
    if (native && rank == 2) {
      L.n0 = ST[0].n;
      L.r_rdist = r2c ? ST[0].is : ST[0].os;
      const int64_t cr = r2c ? ST[0].os : ST[0].is;
      L.c_rdist = cr / 2;
      native = !(cr & 1) && L.r_rdist > 0 && cr > 0 && (L.r_rdist & 1) == 0;
    }
    int64_t vn = 1, vis = 0, vos = 0;
    if (vrank == 1) {
      vn = SV[0].n;
      vis = SV[0].is;
      vos = SV[0].os;
    }
    const int64_t cb = r2c ? vos : vis;
    L.howmany = vn;
    L.r_bdist = r2c ? vis : vos;
    L.c_bdist = cb / 2;
    native = native && !(cb & 1) && (vn <= 1 || (L.r_bdist > 0 && cb > 0 && (L.r_bdist & 1) == 0));
    if (!native) return plan_rdft2_packed(r2c, ST, SV, rRe, cRe, cIm, precision, flags, out);
    L.r_off = rRe;
    L.c_off = cRe / 2;
    lfg::Plan p;
    p.kind = r2c ? lfg::Kind::R2C : lfg::Kind::C2R;
    p.precision = precision;
    p.fwd = r2c;
    p.empty = vn == 0;
    if (p.empty) L.howmany = 1;
    return finish_real(p, L, out);
  }
  if (kind == 2) {
    // r2r (Core/Problem.lean:237-250): real data, one kind per transform dimension
    if (nspec < (size_t)(8 + 3 * (rank + vrank) + rank))
      return fail(LFG_ERR_INVALID, "r2r spec lacks the kinds");
    if (rank < 1) return fail(LFG_ERR_UNSUPPORTED, "rank-0 problems (copies) are not executed");
    std::vector<CDim> T, V;
    std::vector<int> kinds;
    for (int64_t i = 0; i < rank + vrank; ++i) {
      int64_t n, is, os;
      dim(i, &n, &is, &os);
      if (n < 0 || (i < rank && n < 1)) return fail(LFG_ERR_INVALID, "bad dimension");
      if (n > 1 && (is <= 0 || os <= 0)) return fail(LFG_ERR_UNSUPPORTED, "strides must be positive");
      (i < rank ? T : V).push_back(CDim{n, is, os});
    }
    for (int64_t d = 0; d < rank; ++d) {
      const int k = (int)spec[8 + 3 * (rank + vrank) + d];
      if (k < 0 || k > 10) return fail(LFG_ERR_INVALID, "r2r kind outside 0..10");
      kinds.push_back(k);
    }
    if (inRe < 0 || outRe < 0) return fail(LFG_ERR_UNSUPPORTED, "negative offsets");
    return plan_separable(true, T, V, kinds, inRe, outRe, sign, precision, flags, out);
  }
  if (kind != 0) return fail(LFG_ERR_INVALID, "kind must be 0, 1 or 2");
  if (rank < 1) return fail(LFG_ERR_UNSUPPORTED, "rank-0 problems (copies) are not executed");
  // the kernels take interleaved complex data (imaginary part one scalar after the real part)
  // at positive strides of whole complex elements; other layouts (split arrays, strides of
  // either sign) go through dense buffers
  bool interleaved = inIm == inRe + 1 && outIm == outRe + 1 && inRe >= 0 && outRe >= 0 &&
                     !(inRe & 1) && !(outRe & 1);
  for (const auto* Lst : {&ST, &SV})
    for (const SDim& d : *Lst)
      if (d.n > 1 && ((d.is & 1) || (d.os & 1) || d.is <= 0 || d.os <= 0)) interleaved = false;
  if (!interleaved) return plan_c2c_packed(ST, SV, inRe, inIm, outRe, outIm, sign, precision, flags, out);
  if (rank > 1 || vrank > 1) {
    std::vector<CDim> T, V;
    for (const SDim& d : ST) T.push_back(CDim{d.n, d.is / 2, d.os / 2});
    for (const SDim& d : SV) V.push_back(CDim{d.n, d.is / 2, d.os / 2});
    return plan_separable(false, T, V, {}, inRe / 2, outRe / 2, sign, precision, flags, out);
  }
  int64_t n, is, os;
  dim(0, &n, &is, &os);
  int64_t vn = 1, vis = 0, vos = 0;
  if (vrank == 1) dim(1, &vn, &vis, &vos);
  if (vn < 0) return fail(LFG_ERR_INVALID, "negative vector dimension");
  if (vis < 0 || vos < 0 || (vis & 1) || (vos & 1))
    return plan_c2c_packed(ST, SV, inRe, inIm, outRe, outIm, sign, precision, flags, out);
  if (n < 2) return fail(LFG_ERR_UNSUPPORTED, "a transform of one point is a copy");
  lfg::Plan p;
  p.kind = lfg::Kind::C2C;
  p.precision = precision;
  p.fwd = sign < 0;
  p.n = n;
  p.howmany = vn;
  p.empty = vn == 0;
  p.in.offset = inRe / 2;
  p.in.stride = is / 2;
  p.in.dist = vrank == 1 ? vis / 2 : 0;
  p.out.offset = outRe / 2;
  p.out.stride = os / 2;
  p.out.dist = vrank == 1 ? vos / 2 : 0;
  p.radices = lfg::choose_radices(n, precision);
  p.measure = (flags & LFG_MEASURE) != 0;
  return finish_c2c(p, out);
}

static lfg_status lfg_execute_impl(const lfg_plan* plan, const void* in, void* out, void* stream) {
  if (!plan) return fail(LFG_ERR_INVALID, "null plan");
  if (plan->p.empty) return LFG_OK;
  if (!in || !out) return fail(LFG_ERR_INVALID, "null buffer");
  if (!element_aligned(in, plan->p.precision) || !element_aligned(out, plan->p.precision))
    return fail(LFG_ERR_INVALID, "buffers must be aligned to a complex element (16 bytes binary64, 8 bytes binary32)");
  cudaError_t e = lfg::execute_plan(plan->p, in, out, static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "execute");
  return LFG_OK;
}

static lfg_status lfg_execute_host_impl(const lfg_plan* plan, const void* in, void* out) {
  if (!plan) return fail(LFG_ERR_INVALID, "null plan");
  const lfg::Plan& p = plan->p;
  if (p.empty) return LFG_OK;
  if (!in || !out) return fail(LFG_ERR_INVALID, "null buffer");
  const size_t sb = p.precision == 0 ? 8 : 4;
  const size_t ib = (size_t)p.in_span * sb, ob = (size_t)p.out_span * sb;
  cudaError_t e;
  {
    void* mi = mapped_device_ptr(in, ib);
    void* mo = in == out ? mi : mapped_device_ptr(out, ob);
    if (mi && mo && element_aligned(mi, p.precision) && element_aligned(mo, p.precision)) {
      // pinned host buffers: the kernels stream them over NVLink-C2C
      if ((e = lfg::execute_plan(p, mi, mo, 0, true)) != cudaSuccess) return cuda_fail(e, "execute");
      if ((e = cudaStreamSynchronize(0)) != cudaSuccess) return cuda_fail(e, "execute");
      return LFG_OK;
    }
  }
  if (!p.d_host_in) {
    if ((e = cudaMalloc(&p.d_host_in, ib)) != cudaSuccess) return cuda_fail(e, "cudaMalloc");
    if ((e = cudaMalloc(&p.d_host_out, ob)) != cudaSuccess) return cuda_fail(e, "cudaMalloc");
  }
  const bool inplace = in == out;
  void* din = p.d_host_in;
  void* dout = inplace ? p.d_host_in : p.d_host_out;
  if ((e = cudaMemcpy(din, in, ib, cudaMemcpyHostToDevice)) != cudaSuccess)
    return cuda_fail(e, "host-to-device copy");
  // an output span with gaps keeps the caller's values there: bring them along
  const bool dense = p.out.offset == 0 && p.out.stride == 1 && (p.howmany == 1 || p.out.dist == p.n);
  if (!inplace && !dense && (e = cudaMemcpy(dout, out, ob, cudaMemcpyHostToDevice)) != cudaSuccess)
    return cuda_fail(e, "host-to-device copy");
  if ((e = lfg::execute_plan(p, din, dout, 0)) != cudaSuccess) return cuda_fail(e, "execute");
  if ((e = cudaMemcpy(out, dout, ob, cudaMemcpyDeviceToHost)) != cudaSuccess)
    return cuda_fail(e, "device-to-host copy");
  return LFG_OK;
}

void lfg_destroy(lfg_plan* plan) {
  if (!plan) return;
  lfg::free_plan_memory(plan->p);
  delete plan;
}

static lfg_status lfg_set_scale_impl(lfg_plan* plan, double scale) {
  if (!plan) return fail(LFG_ERR_INVALID, "null plan");
  if (!std::isfinite(scale)) return fail(LFG_ERR_INVALID, "scale must be finite");
  lfg::Plan& p = plan->p;
  if (p.kind != lfg::Kind::C2C) return fail(LFG_ERR_UNSUPPORTED, "scaling applies to complex plans");
  lfg::Plan* target = p.stages.empty() ? &p : p.stages.back().plan.get();
  if (target->generic) {
    target->gen.scale = scale;
  } else if (target->chirp_bwd) {
    lfg::Plan& b = *target->chirp_bwd;
    if (b.ngroups >= 1) b.groups[b.ngroups - 1].scale = scale / (double)target->chirp.L;
  } else if (!p.stages.empty()) {
    lfg::Plan& last = *p.stages.back().plan;
    if (last.ngroups >= 1) last.groups[last.ngroups - 1].scale = scale;
  } else if (p.ngroups >= 1) {
    p.groups[p.ngroups - 1].scale = scale;
  }
  return LFG_OK;
}

static lfg_status lfg_device_status_impl(const lfg_plan* plan) {
  if (!plan) return fail(LFG_ERR_INVALID, "null plan");
  const lfg::Plan& p = plan->p;
  if (!p.d_status) return LFG_OK;
  int v = 0;
  cudaError_t e = cudaMemcpy(&v, p.d_status, sizeof v, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, "status read");
  if (v) {
    cudaMemset(p.d_status, 0, sizeof v);
    return fail(LFG_ERR_TIMEOUT, "a bounded device-side wait gave up (bulk copy not completed)");
  }
  return LFG_OK;
}

static lfg_status lfg_get_plan_info_impl(const lfg_plan* plan, lfg_plan_info* info) {
  if (!plan || !info) return fail(LFG_ERR_INVALID, "null argument");
  const lfg::Plan& p = plan->p;
  std::memset(info, 0, sizeof *info);
  info->n = p.n;
  info->howmany = p.howmany;
  info->sign = p.fwd ? -1 : 1;
  info->precision = p.precision;
  info->npass = (int)p.radices.size();
  info->ngroups = p.ngroups;
  for (size_t i = 0; i < p.radices.size() && i < 24; ++i) info->radices[i] = p.radices[i];
  info->in_bytes = p.in_span * (p.precision == 0 ? 8 : 4);
  info->out_bytes = p.out_span * (p.precision == 0 ? 8 : 4);
  info->flops = p.flops;
  info->cluster_ctas = p.cluster ? p.cluster_args.S : 0;
  info->direct_groups = (p.direct_variant[0] >= 0) + (p.direct_variant[1] >= 0);
  info->small_kernel = p.small_grid ? 1 : 0;
  return LFG_OK;
}

static lfg_status lfg_plan_ragged_impl(const int64_t* sizes, size_t count, const int64_t* in_offsets,
                           const int64_t* out_offsets, int sign, lfg_precision precision,
                           unsigned flags, const lfg_ragged_tuning* tuning, lfg_ragged** out) {
  if (!out) return fail(LFG_ERR_INVALID, "null output handle");
  *out = nullptr;
  if (!sizes && count) return fail(LFG_ERR_INVALID, "null sizes");
  if (sign != -1 && sign != 1) return fail(LFG_ERR_INVALID, "sign must be -1 or +1");
  if (precision != LFG_F64) return fail(LFG_ERR_UNSUPPORTED, "precision not supported yet");
  lfg::RaggedPlan r;
  r.precision = precision;
  r.fwd = sign < 0;
  r.empty = count == 0;
  r.use_graph = !(flags & LFG_NO_GRAPH);
  r.per_size_mode = (flags & LFG_PER_SIZE) != 0;
  r.per_size_concurrent = r.per_size_mode && (flags & LFG_PER_SIZE_CONCURRENT) != 0;
  r.sizes.assign(sizes, sizes + count);
  int64_t acc_in = 0, acc_out = 0;
  for (size_t i = 0; i < count; ++i) {
    const int64_t n = sizes[i];
    if (n < 2 || n > ((int64_t)1 << 24) || !smooth13(n))
      return fail(LFG_ERR_UNSUPPORTED, "size " + std::to_string(n) + " must be 13-smooth in 2..2^24");
    const int64_t io = in_offsets ? in_offsets[i] : acc_in;
    const int64_t oo = out_offsets ? out_offsets[i] : acc_out;
    if (io < 0 || oo < 0) return fail(LFG_ERR_INVALID, "negative offset");
    r.in_off.push_back(io);
    r.out_off.push_back(oo);
    r.in_span = std::max(r.in_span, io + n);
    r.out_span = std::max(r.out_span, oo + n);
    acc_in += n;
    acc_out += n;
  }
  {
    // the outputs tile [0, out_span) exactly when sorted offsets leave no gap
    std::vector<std::pair<int64_t, int64_t>> iv;
    for (size_t i = 0; i < count; ++i) iv.push_back({r.out_off[i], sizes[i]});
    std::sort(iv.begin(), iv.end());
    int64_t pos = 0;
    bool dense = true;
    for (auto& q : iv) {
      if (q.first != pos) { dense = false; break; }
      pos += q.second;
    }
    r.out_dense = dense && pos == r.out_span;
  }
  lfg::RaggedOptions opt;
  opt.tile_target = tile_target();
  if (tuning) {
    if (tuning->tile_target >= 16) opt.tile_target = tuning->tile_target;
    if (tuning->single_max >= 2) opt.single_max = tuning->single_max;
    if (tuning->block_shape < 0 || tuning->block_shape >= lfg::kRaggedVariants)
      return fail(LFG_ERR_INVALID, "bad block shape");
    opt.variant = tuning->block_shape;
    for (int j = 0; j < tuning->n_over; ++j) {
      const int np = tuning->over_npass[j];
      if (np < 1 || np > lfg::kMaxPass) return fail(LFG_ERR_INVALID, "bad override pass count");
      opt.radices[tuning->over_n[j]] =
          std::vector<int>(tuning->over_radices + 24 * j, tuning->over_radices + 24 * j + np);
    }
  }
  opt.single_max = std::min<int64_t>(opt.single_max, lfg::max_single_group(precision));
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  r.device = dev;
  if (!r.empty) {
    e = lfg::prepare_group_kernels_f64();
    if (e != cudaSuccess) return cuda_fail(e, "kernel set-up");
    if (flags & LFG_MEASURE) {
      std::string tm = lfg::tune_ragged(r, opt);
      if (!tm.empty()) return fail(LFG_ERR_CUDA, tm);
    }
    r.options = opt;
    std::string msg = lfg::build_ragged(r, opt);
    if (!msg.empty()) {
      lfg::free_ragged(r);
      return fail(LFG_ERR_UNSUPPORTED, msg);
    }
  }
  lfg_ragged* h = new (std::nothrow) lfg_ragged;
  if (!h) {
    lfg::free_ragged(r);
    return fail(LFG_ERR_NOMEM, "host allocation");
  }
  h->r = std::move(r);
  *out = h;
  return LFG_OK;
}

static lfg_status lfg_execute_ragged_impl(const lfg_ragged* plan, const void* in, void* out, void* stream) {
  if (!plan) return fail(LFG_ERR_INVALID, "null plan");
  if (plan->r.empty) return LFG_OK;
  if (!in || !out) return fail(LFG_ERR_INVALID, "null buffer");
  if (in == out) return fail(LFG_ERR_UNSUPPORTED, "ragged batches run out of place");
  if (!element_aligned(in, plan->r.precision) || !element_aligned(out, plan->r.precision))
    return fail(LFG_ERR_INVALID, "buffers must be aligned to a complex element (16 bytes binary64, 8 bytes binary32)");
  cudaError_t e = lfg::execute_ragged(plan->r, in, out, static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "execute ragged");
  return LFG_OK;
}

static lfg_status lfg_execute_ragged_host_impl(const lfg_ragged* plan, const void* in, void* out) {
  if (!plan) return fail(LFG_ERR_INVALID, "null plan");
  const lfg::RaggedPlan& r = plan->r;
  if (r.empty) return LFG_OK;
  if (!in || !out || in == out) return fail(LFG_ERR_INVALID, "bad buffers");
  const size_t es = r.precision == 0 ? 16 : 8;
  const size_t ib = (size_t)r.in_span * es, ob = (size_t)r.out_span * es;
  cudaError_t e;
  {
    void* mi = mapped_device_ptr(in, ib);
    void* mo = mapped_device_ptr(out, ob);
    if (mi && mo && element_aligned(mi, r.precision) && element_aligned(mo, r.precision)) {
      // pinned host buffers: the kernel streams them over NVLink-C2C
      if ((e = lfg::execute_ragged_mapped(r, mi, mo, 0)) != cudaSuccess) return cuda_fail(e, "execute ragged");
      if ((e = cudaStreamSynchronize(0)) != cudaSuccess) return cuda_fail(e, "execute ragged");
      return LFG_OK;
    }
  }
  if (!r.d_host_in) {
    if ((e = cudaMalloc(&r.d_host_in, ib)) != cudaSuccess) return cuda_fail(e, "cudaMalloc");
    if ((e = cudaMalloc(&r.d_host_out, ob)) != cudaSuccess) return cuda_fail(e, "cudaMalloc");
  }
  if ((e = cudaMemcpy(r.d_host_in, in, ib, cudaMemcpyHostToDevice)) != cudaSuccess)
    return cuda_fail(e, "host-to-device copy");
  // an output span with gaps keeps the caller's values there: bring them along
  if (!r.out_dense && (e = cudaMemcpy(r.d_host_out, out, ob, cudaMemcpyHostToDevice)) != cudaSuccess)
    return cuda_fail(e, "host-to-device copy");
  if ((e = lfg::execute_ragged(r, r.d_host_in, r.d_host_out, 0)) != cudaSuccess)
    return cuda_fail(e, "execute ragged");
  if ((e = cudaMemcpy(out, r.d_host_out, ob, cudaMemcpyDeviceToHost)) != cudaSuccess)
    return cuda_fail(e, "device-to-host copy");
  return LFG_OK;
}

void lfg_destroy_ragged(lfg_ragged* plan) {
  if (!plan) return;
  lfg::free_ragged(plan->r);
  delete plan;
}

static lfg_status lfg_get_ragged_info_impl(const lfg_ragged* plan, lfg_ragged_info* info) {
  if (!plan || !info) return fail(LFG_ERR_INVALID, "null argument");
  const lfg::RaggedPlan& r = plan->r;
  std::memset(info, 0, sizeof *info);
  info->count = (int64_t)r.sizes.size();
  info->classes = (int64_t)r.class_n.size();
  info->items = (int64_t)r.items_host.size();
  info->grid = r.launch.grid;
  info->smem_bytes = (int64_t)r.launch.smem;
  int64_t launches = 1;
  if (r.per_size_mode) {
    launches = 0;
    for (const auto& L : r.per_size) launches += L.ngroups;
  }
  info->launches = r.empty ? 0 : launches;
  const int64_t es = r.precision == 0 ? 16 : 8;
  info->in_bytes = r.in_span * es;
  info->out_bytes = r.out_span * es;
  for (int64_t n : r.sizes) info->points += n;
  info->flops = r.flops;
  info->tile_target = r.options.tile_target;
  info->single_max = std::min(r.options.single_max, lfg::ragged_max_single_group());
  info->block_shape = r.options.variant;
  return LFG_OK;
}

static lfg_status lfg_get_ragged_radices_impl(const lfg_ragged* plan, int64_t n, int* radices, int* npass) {
  if (!plan || !radices || !npass) return fail(LFG_ERR_INVALID, "null argument");
  const lfg::RaggedPlan& r = plan->r;
  *npass = 0;
  for (size_t c = 0; c < r.class_n.size(); ++c)
    if (r.class_n[c] == n) {
      *npass = (int)r.class_radices[c].size();
      for (int i = 0; i < *npass; ++i) radices[i] = r.class_radices[c][i];
    }
  return LFG_OK;
}

const char* lfg_strerror(lfg_status s) {
  switch (s) {
    case LFG_OK: return "ok";
    case LFG_ERR_UNSUPPORTED: return "problem not supported";
    case LFG_ERR_INVALID: return "invalid argument";
    case LFG_ERR_CUDA: return "CUDA error";
    case LFG_ERR_NOMEM: return "out of memory";
    case LFG_ERR_TIMEOUT: return "device wait timed out";
  }
  return "unknown status";
}

const char* lfg_last_error(void) { return g_last_error.c_str(); }

static lfg_status lfg_cos_sin_table_impl(uint64_t n, double* out) {
  if (!out || n == 0) return fail(LFG_ERR_INVALID, "bad arguments");
  std::vector<double> t = lfg::cos_sin_2pi_table(n);
  std::memcpy(out, t.data(), t.size() * sizeof(double));
  return LFG_OK;
}

static lfg_status lfg_plan_layout_impl(size_t n, lfg_precision precision, int* radices,
                                       int* npass, int* first_group) {
  if (!radices || !npass || !first_group) return fail(LFG_ERR_INVALID, "null output");
  if (precision != LFG_F64 && precision != LFG_F32) return fail(LFG_ERR_INVALID, "bad precision");
  if (n < 2 || n > ((size_t)1 << 24)) return fail(LFG_ERR_UNSUPPORTED, "size outside 2..2^24");
  if (!smooth13((int64_t)n))
    return fail(LFG_ERR_UNSUPPORTED, "sizes with a prime factor above 13 take the generic engine");
  std::vector<int> rs = lfg::choose_radices((int64_t)n, precision);
  const int64_t single = precision == 0 ? single_max_default() : lfg::kF32SingleGroupMax;
  const int split = lfg::choose_split((int64_t)n, rs, single, precision, true);
  if (split < 0 || (int)rs.size() > lfg::kMaxPass)
    return fail(LFG_ERR_UNSUPPORTED, "no two-group split for this size");
  std::copy(rs.begin(), rs.end(), radices);
  *npass = (int)rs.size();
  *first_group = split;
  return LFG_OK;
}

static lfg_status lfg_shard_ragged_impl(const int64_t* sizes, size_t count, int nshards,
                                        int* shard, double* cost) {
  if ((!sizes || !shard) && count) return fail(LFG_ERR_INVALID, "null array");
  if (nshards < 1) return fail(LFG_ERR_INVALID, "nshards must be >= 1");
  // cost of a transform: its codelet operations (the binary64 kernels are bound by them);
  // sizes the fast engine does not cover count 5 n log2 n
  std::vector<double> c(count);
  std::map<int64_t, double> memo;
  for (size_t i = 0; i < count; ++i) {
    const int64_t n = sizes[i];
    if (n < 1) return fail(LFG_ERR_INVALID, "sizes must be >= 1");
    auto it = memo.find(n);
    if (it == memo.end()) {
      double v = 5.0 * (double)n * std::log2((double)std::max<int64_t>(2, n));
      if (n >= 2 && n <= ((int64_t)1 << 24) && smooth13(n))
        v = lfg::plan_ops(n, lfg::choose_radices(n, 0));
      it = memo.emplace(n, v).first;
    }
    c[i] = it->second;
  }
  // longest processing time first: each transform, largest first (ties by index), to the
  // least loaded shard (ties to the lower shard) -- deterministic on every rank
  std::vector<size_t> order(count);
  for (size_t i = 0; i < count; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return c[a] > c[b]; });
  std::vector<double> load(nshards, 0.0);
  for (size_t i : order) {
    const int s = (int)(std::min_element(load.begin(), load.end()) - load.begin());
    shard[i] = s;
    load[s] += c[i];
  }
  if (cost) std::copy(load.begin(), load.end(), cost);
  return LFG_OK;
}

static lfg_status lfg_wisdom_import_impl(const char* path) {
  if (!path) return fail(LFG_ERR_INVALID, "null path");
  if (!lfg::wisdom_import(path)) return fail(LFG_ERR_INVALID, std::string("cannot read ") + path);
  return LFG_OK;
}

static lfg_status lfg_wisdom_export_impl(const char* path) {
  if (!path) return fail(LFG_ERR_INVALID, "null path");
  if (!lfg::wisdom_export(path)) return fail(LFG_ERR_INVALID, std::string("cannot write ") + path);
  return LFG_OK;
}

void lfg_wisdom_forget(void) { lfg::wisdom_forget(); }

size_t lfg_wisdom_count(void) { return lfg::wisdom_size(); }


// The exported entry points: every C++ exception (host allocation failures above all) is
// turned into a status here, so none crosses the C ABI.

lfg_status lfg_plan_1d(size_t n, int sign, size_t howmany, lfg_precision precision,
                       unsigned flags, lfg_plan** out) {
  return guarded([&] { return lfg_plan_1d_impl(n, sign, howmany, precision, flags, out); });
}

lfg_status lfg_plan_r2c(size_t n, size_t howmany, lfg_precision precision, unsigned flags,
                        lfg_plan** out) {
  return guarded([&] { return lfg_plan_r2c_impl(n, howmany, precision, flags, out); });
}

lfg_status lfg_plan_c2r(size_t n, size_t howmany, lfg_precision precision, unsigned flags,
                        lfg_plan** out) {
  return guarded([&] { return lfg_plan_c2r_impl(n, howmany, precision, flags, out); });
}

lfg_status lfg_plan_r2c_2d(size_t n0, size_t n1, size_t howmany, lfg_precision precision,
                           unsigned flags, lfg_plan** out) {
  return guarded([&] { return lfg_plan_r2c_2d_impl(n0, n1, howmany, precision, flags, out); });
}

lfg_status lfg_plan_c2r_2d(size_t n0, size_t n1, size_t howmany, lfg_precision precision,
                           unsigned flags, lfg_plan** out) {
  return guarded([&] { return lfg_plan_c2r_2d_impl(n0, n1, howmany, precision, flags, out); });
}

lfg_status lfg_plan_r2r(size_t n, int kind, size_t howmany, lfg_precision precision,
                        unsigned flags, lfg_plan** out) {
  return guarded([&] { return lfg_plan_r2r_impl(n, kind, howmany, precision, flags, out); });
}

lfg_status lfg_plan_1d_radices(size_t n, int sign, size_t howmany, lfg_precision precision,
                               const int* radices, int npass, lfg_plan** out) {
  return guarded([&] { return lfg_plan_1d_radices_impl(n, sign, howmany, precision, radices, npass, out); });
}

lfg_status lfg_plan_spec(const double* spec, size_t nspec, lfg_precision precision,
                         unsigned flags, lfg_plan** out) {
  return guarded([&] { return lfg_plan_spec_impl(spec, nspec, precision, flags, out); });
}

lfg_status lfg_execute(const lfg_plan* plan, const void* in, void* out, void* stream) {
  return guarded([&] { return lfg_execute_impl(plan, in, out, stream); });
}

lfg_status lfg_execute_host(const lfg_plan* plan, const void* in, void* out) {
  return guarded([&] { return lfg_execute_host_impl(plan, in, out); });
}

lfg_status lfg_set_scale(lfg_plan* plan, double scale) {
  return guarded([&] { return lfg_set_scale_impl(plan, scale); });
}

lfg_status lfg_device_status(const lfg_plan* plan) {
  return guarded([&] { return lfg_device_status_impl(plan); });
}

lfg_status lfg_get_plan_info(const lfg_plan* plan, lfg_plan_info* info) {
  return guarded([&] { return lfg_get_plan_info_impl(plan, info); });
}

lfg_status lfg_plan_ragged(const int64_t* sizes, size_t count, const int64_t* in_offsets,
                           const int64_t* out_offsets, int sign, lfg_precision precision,
                           unsigned flags, const lfg_ragged_tuning* tuning, lfg_ragged** out) {
  return guarded([&] {
    return lfg_plan_ragged_impl(sizes, count, in_offsets, out_offsets, sign, precision, flags,
                                tuning, out);
  });
}

lfg_status lfg_execute_ragged(const lfg_ragged* plan, const void* in, void* out, void* stream) {
  return guarded([&] { return lfg_execute_ragged_impl(plan, in, out, stream); });
}

lfg_status lfg_execute_ragged_host(const lfg_ragged* plan, const void* in, void* out) {
  return guarded([&] { return lfg_execute_ragged_host_impl(plan, in, out); });
}

lfg_status lfg_get_ragged_info(const lfg_ragged* plan, lfg_ragged_info* info) {
  return guarded([&] { return lfg_get_ragged_info_impl(plan, info); });
}

lfg_status lfg_get_ragged_radices(const lfg_ragged* plan, int64_t n, int* radices, int* npass) {
  return guarded([&] { return lfg_get_ragged_radices_impl(plan, n, radices, npass); });
}

lfg_status lfg_cos_sin_table(uint64_t n, double* out) {
  return guarded([&] { return lfg_cos_sin_table_impl(n, out); });
}

lfg_status lfg_shard_ragged(const int64_t* sizes, size_t count, int nshards, int* shard,
                            double* cost) {
  return guarded([&] { return lfg_shard_ragged_impl(sizes, count, nshards, shard, cost); });
}

lfg_status lfg_plan_layout(size_t n, lfg_precision precision, int* radices, int* npass,
                           int* first_group) {
  return guarded([&] { return lfg_plan_layout_impl(n, precision, radices, npass, first_group); });
}

lfg_status lfg_wisdom_import(const char* path) {
  return guarded([&] { return lfg_wisdom_import_impl(path); });
}

lfg_status lfg_wisdom_export(const char* path) {
  return guarded([&] { return lfg_wisdom_export_impl(path); });
}
}  // extern "C"
