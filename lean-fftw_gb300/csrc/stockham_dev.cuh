// Device-side building blocks of the Stockham kernels (pass, tile copy, tile driver), for
// binary64 (T = double) and binary32 (T = float).
//
// Each butterfly is a generated codelet (generated/codelets_f{64,32}.cuh) evaluated with
// explicitly rounded IEEE operations, so each binary64 pass performs exactly the operations
// of lean-fftw's reference pass (`LeanFFTW/Gen/Stockham.lean:263-284`); stockham.h explains
// why grouping passes over sub-problems preserves this.  The binary32 passes run the same
// operation DAGs in binary32, with twiddles rounded from the binary64 tables; passes marked
// `comp` multiply by twiddles held as two binary32 parts (hi + lo) with compensated products.
#pragma once
#include <cuda_runtime.h>

#include "generated/codelets_f32.cuh"
#include "generated/codelets_f64.cuh"
#include "kernels.h"
#include "stockham.h"

namespace lfg {
namespace dev {

template <class T>
struct Prec;

// 1.0 and -0.0 for the binary64 codelets' fused forms of a + b and a * b (generated
// codelets: a*1 + b and a*b + (-0) round exactly as the add and the multiply).  Each pass
// reads them with an opaque non-coherent load (inline PTX, served by L1), so the compiler
// cannot fold the fused forms back into DADD/DMUL.
static __device__ double lfg_fma_units[2] = {1.0, -0.0};

template <>
struct Prec<double> {
  using C = double2;
  template <bool F, int R, bool W>
  using Bfly = BflyD<F, R, W>;
  static __device__ __forceinline__ C mk(double a, double b) { return make_double2(a, b); }
  static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
  static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
  static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
  static __device__ __forceinline__ double fma(double a, double b, double c) { return __fma_rn(a, b, c); }
  static __device__ __forceinline__ void units(double& one, double& nz) {
    const size_t a = __cvta_generic_to_global(lfg_fma_units);
    asm volatile("ld.global.nc.f64 %0, [%1];" : "=d"(one) : "l"(a));
    asm volatile("ld.global.nc.f64 %0, [%1+8];" : "=d"(nz) : "l"(a));
  }
};

template <>
struct Prec<float> {
  using C = float2;
  template <bool F, int R, bool W>
  using Bfly = BflyF<F, R, W>;
  static __device__ __forceinline__ C mk(float a, float b) { return make_float2(a, b); }
  static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
  static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
  static __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
  static __device__ __forceinline__ float fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
  static __device__ __forceinline__ void units(float& one, float& nz) {   // unused by binary32
    one = 1.0f;
    nz = -0.0f;
  }
};


// Within a sub-problem, one padding element after every 16: a Stockham pass stores its
// outputs at stride R (up to 16 elements = 128 or 256 bytes) between neighbouring threads,
// which would put a whole warp on one bank; with the padding the stride is 17 elements.
// Sub-problems start sub_pitch(M) elements apart (stockham.h).
__device__ __forceinline__ int spad(int i) { return i + (i >> 4); }

// n / d for 0 <= n < 2^31 with the plan's FastDiv of d (stockham.h).
__device__ __forceinline__ int fdiv(int n, const FastDiv& f) {
  return (int)((__umulhi(f.m, (unsigned)n) + (unsigned)n) >> f.l);
}

// Destination of a pass's outputs: the next shared-memory tile buffer (padded layout).  A
// pass takes it as a policy object (row(c): start of sub-problem c; put: one output).
template <class T>
struct SmemOut {
  typename Prec<T>::C* dst;
  int pitch;
  __device__ __forceinline__ typename Prec<T>::C* row(int c) const { return dst + c * pitch; }
  __device__ __forceinline__ void put(typename Prec<T>::C* row, int i, typename Prec<T>::C v) const {
    row[spad(i)] = v;
  }
};

// One pass over the C sub-problems of a tile: src is a tile buffer in shared memory (padded
// unless SRCPAD is false, as for a stage buffer a bulk copy filled); outputs go to `out`.
// MODE 0: untwiddled; 1: twiddled codelet (table twiddles); 2: compensated twiddle products
// with (hi, lo) binary32 twiddles, then the untwiddled codelet.
// sub0: index within its line of the tile's first sub-problem (second group), else -1.
//
// Twiddle tables hold (re, im) pairs (interleave_tables): one vector load per twiddle (6 %
// faster for binary32 1024-point lines; the binary64 kernels are unchanged).  Computing the
// padded shared-memory addresses incrementally, where spad is affine in r, measured 2-5 %
// slower for the binary64 kernels, so every address is formed with spad.
template <class T, bool FWD, int R, int MODE, bool SRCPAD, class Out>
__device__ __forceinline__ void pass_t(const typename Prec<T>::C* __restrict__ src,
                                       const Out& out, int C, int M,
                                       const PassDesc& pd, int sub0, int nsub,
                                       const FastDiv fd_nsub) {
  using P = Prec<T>;
  using Cx = typename P::C;
  constexpr bool TW = MODE == 1;
  const int MR = M / R;
  const int nb = C * MR;
  const int ns = pd.ns_loc;
  const Cx* __restrict__ tw = static_cast<const Cx*>(pd.tw);
  const int nsg = pd.ns_g;             // < 2^24: products with r stay in int
  const FastDiv fd_mr = pd.fd_mr, fd_ns = pd.fd_ns;
  const int PM = sub_pitch(M);
  T one, nz;
  P::units(one, nz);
  for (int q = threadIdx.x; q < nb; q += blockDim.x) {
    const int c = fdiv(q, fd_mr);
    const int j = q - c * MR;
    T x[TW ? 4 * R - 2 : 2 * R];
    T y[2 * R];
    const Cx* sc = src + (SRCPAD ? c * PM : c * M);
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int si = j + r * MR;
      const Cx v = sc[SRCPAD ? spad(si) : si];
      x[2 * r] = v.x;
      x[2 * r + 1] = v.y;
    }
    const int b = fdiv(j, fd_ns);
    const int k = j - b * ns;
    // table index of the twiddle: k (one group, or the first), or, in the second group,
    // m * ns_loc + k with m the sub-problem index within its line (the planner stores those
    // tables transposed; tiles may straddle lines, so m wraps at nsub)
    int64_t kg = k;
    if (sub0 >= 0) {
      const int t = sub0 + c;
      kg = (int64_t)(t - fdiv(t, fd_nsub) * nsub) * ns + k;
    }
    if (MODE == 1) {
      const Cx* __restrict__ w = tw + kg;
#pragma unroll
      for (int r = 0; r < R - 1; ++r) {
        const Cx v = __ldg(w + r * nsg);
        x[2 * R + 2 * r] = v.x;
        x[2 * R + 2 * r + 1] = v.y;
      }
    } else if (MODE == 2) {
      // w = (wr_hi + wr_lo) + i (wi_hi + wi_lo); the lo table follows the hi table
      const Cx* __restrict__ wh = tw + kg;
      const Cx* __restrict__ wl = wh + (int64_t)(R - 1) * nsg;
#pragma unroll
      for (int r = 1; r < R; ++r) {
        const Cx h = __ldg(wh + (r - 1) * nsg), l = __ldg(wl + (r - 1) * nsg);
        const T wrh = h.x, wih = h.y, wrl = l.x, wil = l.y;
        const T a = x[2 * r], bi = x[2 * r + 1];
        const T cr = P::fma(a, wrl, -P::mul(bi, wil));          // small correction terms
        const T ci = P::fma(a, wil, P::mul(bi, wrl));
        x[2 * r] = P::fma(a, wrh, P::fma(-bi, wih, cr));
        x[2 * r + 1] = P::fma(a, wih, P::fma(bi, wrh, ci));
      }
    }
    P::template Bfly<FWD, R, TW>::run(x, y, one, nz);
    const int d0 = b * ns * R + k;
    Cx* dc = out.row(c);
#pragma unroll
    for (int r = 0; r < R; ++r) out.put(dc, d0 + r * ns, P::mk(y[2 * r], y[2 * r + 1]));
  }
}

template <class T, bool FWD, bool SRCPAD = true, class Out>
__device__ __forceinline__ void run_pass_to(const typename Prec<T>::C* src, const Out& out,
                                            int C, int M, const PassDesc& pd, int sub0, int nsub,
                                            const FastDiv fd_nsub) {
#define LFG_PASS_CASE(RR)                                                                        \
  case RR:                                                                                       \
    if (!pd.tw) pass_t<T, FWD, RR, 0, SRCPAD>(src, out, C, M, pd, sub0, nsub, fd_nsub);          \
    else if (sizeof(T) == 4 && pd.comp)                                                          \
      pass_t<T, FWD, RR, 2, SRCPAD>(src, out, C, M, pd, sub0, nsub, fd_nsub);                    \
    else pass_t<T, FWD, RR, 1, SRCPAD>(src, out, C, M, pd, sub0, nsub, fd_nsub);                 \
    break;
  switch (pd.R) {
    LFG_PASS_CASE(2)
    LFG_PASS_CASE(3)
    LFG_PASS_CASE(4)
    LFG_PASS_CASE(5)
    LFG_PASS_CASE(6)
    LFG_PASS_CASE(7)
    LFG_PASS_CASE(8)
    LFG_PASS_CASE(9)
    LFG_PASS_CASE(10)
    LFG_PASS_CASE(11)
    LFG_PASS_CASE(12)
    LFG_PASS_CASE(13)
    LFG_PASS_CASE(14)
    LFG_PASS_CASE(15)
    LFG_PASS_CASE(16)
    default: break;   // rejected by the planner
  }
#undef LFG_PASS_CASE
}

// A pass from one shared-memory tile buffer to another.
template <class T, bool FWD, bool SRCPAD = true>
__device__ __forceinline__ void run_pass_t(const typename Prec<T>::C* src, typename Prec<T>::C* dst,
                                           int C, int M, const PassDesc& pd, int sub0, int nsub,
                                           const FastDiv fd_nsub) {
  run_pass_to<T, FWD, SRCPAD>(src, SmemOut<T>{dst, sub_pitch(M)}, C, M, pd, sub0, nsub, fd_nsub);
}

// Line bases (complex-element offsets of each line) of the two tile sources: evenly strided
// lines of a batched plan, or a list of per-transform offsets of a ragged batch.
struct StridedLines {
  int64_t in_line, out_line;
  __device__ int64_t in(int64_t line) const { return line * in_line; }
  __device__ int64_t out(int64_t line) const { return line * out_line; }
  // line pitch of a side (lets a whole tile of back-to-back lines copy as one range)
  __device__ int64_t pitch(bool load) const { return load ? in_line : out_line; }
};

struct ListedLines {
  const int64_t* __restrict__ in_off;
  const int64_t* __restrict__ out_off;
  int64_t first;
  __device__ int64_t in(int64_t line) const { return __ldg(in_off + first + line); }
  __device__ int64_t out(int64_t line) const { return __ldg(out_off + first + line); }
  __device__ int64_t pitch(bool) const { return -1; }
};

// Copy a tile between global memory and a shared-memory tile buffer; the loop order makes
// consecutive threads touch consecutive global addresses (elements of a sub-problem when
// they are contiguous, else neighbouring sub-problems).
template <class T, bool LOAD, class Lines>
__device__ __forceinline__ void copy_tile(typename Prec<T>::C* tile, const typename Prec<T>::C* gin,
                                          typename Prec<T>::C* gout, const GroupDesc& g,
                                          const Lines& lines, int64_t s0, int C) {
  using P = Prec<T>;
  // descriptor fields in registers: the loops below store through generic pointers, after
  // which fields read through a reference would be loaded again every iteration
  const int64_t sub_st = LOAD ? g.in_sub : g.out_sub;
  const int64_t elem_st = LOAD ? g.in_elem : g.out_elem;
  const int M = g.M;
  const int nsub = g.nsub;
  const int gC = g.C;
  const FastDiv fd_m = g.fd_m, fd_c = g.fd_c, fd_nsub = g.fd_nsub;
  const Lines L = lines;
  const int n = C * M;
  const bool elem_fast = (elem_st == 1);
  if (elem_fast && nsub == 1 && L.pitch(LOAD) == M && g.unit_scale) {
    // back-to-back lines: the tile is one contiguous range of global memory
    const int64_t base = (LOAD ? L.in(s0) : L.out(s0));
    const int PM = sub_pitch(M);
    for (int idx = threadIdx.x; idx < n; idx += blockDim.x) {
      const int c = fdiv(idx, fd_m);
      const int t = c * PM + spad(idx - c * M);
      if (LOAD) tile[t] = gin[base + idx];
      else gout[base + idx] = tile[t];
    }
    return;
  }
  // line and in-line index of the tile's first sub-problem (one 64-bit division per tile)
  const int64_t line0 = s0 / nsub;
  const int sub0 = (int)(s0 - line0 * nsub);
  // strided sub-problems: neighbouring threads take neighbouring sub-problems, over the full
  // tile width g.C (a partial last tile skips the missing columns).  Each thread walks its
  // elements with running (sub-problem, element) indices -- one division per tile -- and a
  // tile inside one line reads that line's base once.
  const int nn = elem_fast ? n : gC * M;
  const bool unit = g.unit_scale != 0;
  const T sc = sizeof(T) == 4 ? (T)g.scale_f32 : (T)g.scale;
  const int PM = sub_pitch(M);
  const int S = blockDim.x;
  int c, i, dc, di;
  if (elem_fast) {
    c = fdiv(threadIdx.x, fd_m);
    i = threadIdx.x - c * M;
    dc = fdiv(S, fd_m);
    di = S - dc * M;
  } else {
    i = fdiv(threadIdx.x, fd_c);
    c = threadIdx.x - i * gC;
    di = fdiv(S, fd_c);
    dc = S - di * gC;
  }
  const bool one_line = sub0 + C <= nsub;
  const int64_t base0 = one_line ? (LOAD ? L.in(line0) : L.out(line0)) + (int64_t)sub0 * sub_st : 0;
  for (int idx = threadIdx.x; idx < nn; idx += S) {
    if (c < C) {
      int64_t a;
      if (one_line) {
        a = base0 + (int64_t)c * sub_st + (int64_t)i * elem_st;
      } else {
        const int t = sub0 + c;
        const int ql = fdiv(t, fd_nsub);
        const int64_t line = line0 + ql;
        const int64_t sub = t - ql * nsub;
        a = (LOAD ? L.in(line) : L.out(line)) + sub * sub_st + (int64_t)i * elem_st;
      }
      if (LOAD) {
        tile[c * PM + spad(i)] = gin[a];
      } else if (unit) {
        gout[a] = tile[c * PM + spad(i)];
      } else {
        const auto v = tile[c * PM + spad(i)];
        gout[a] = P::mk(P::mul(v.x, sc), P::mul(v.y, sc));
      }
    }
    c += dc;
    i += di;
    if (elem_fast) {
      if (i >= M) {
        i -= M;
        ++c;
      }
    } else if (c >= gC) {
      c -= gC;
      ++i;
    }
  }
}

// Run every pass of group g on a tile of C sub-problems held in shared-memory buffer A
// (B is the ping-pong partner); returns the buffer holding the result.
template <class T, bool FWD>
__device__ __forceinline__ typename Prec<T>::C* run_passes(const GroupDesc& g,
                                                           typename Prec<T>::C* A,
                                                           typename Prec<T>::C* B, int C,
                                                           int64_t msub0) {
  const int npass = g.npass;
  const int sub0 = msub0 >= 0 ? (int)(msub0 % g.nsub) : -1;
  const FastDiv fd_nsub = g.fd_nsub;
  for (int t = 0; t < npass; ++t) {
    run_pass_t<T, FWD>(A, B, C, g.M, g.pass[t], sub0, g.nsub, fd_nsub);
    __syncthreads();
    auto tmp = A;
    A = B;
    B = tmp;
  }
  return A;
}

// Destination of a last pass that writes global memory directly (the ragged kernel), for
// groups whose output sub-problems are contiguous runs (out_elem == 1): sub-problem c of a tile
// whose first sub-problem is (line0, sub0) starts at this address.  The last pass's outputs of
// one index r are consecutive elements across consecutive threads, so the stores coalesce.
template <class T, class Lines>
struct GlobalRows {
  typename Prec<T>::C* dst;
  FastDiv fd_nsub;       // the group's fields it needs, held by value (registers)
  int nsub;
  int64_t out_sub;
  Lines lines;
  int64_t line0;
  int sub0;
  __device__ __forceinline__ GlobalRows(typename Prec<T>::C* d, const GroupDesc& g, Lines l,
                                        int64_t l0, int s0)
      : dst(d), fd_nsub(g.fd_nsub), nsub(g.nsub), out_sub(g.out_sub), lines(l), line0(l0), sub0(s0) {}
  __device__ __forceinline__ typename Prec<T>::C* row(int c) const {
    const int t = sub0 + c;
    const int ql = fdiv(t, fd_nsub);
    return dst + lines.out(line0 + ql) + (int64_t)(t - ql * nsub) * out_sub;
  }
  __device__ __forceinline__ void put(typename Prec<T>::C* row, int i, typename Prec<T>::C v) const {
    row[i] = v;
  }
};

// Load C sub-problems starting at s0, run every pass of group g in shared memory, store.
// (Letting the last pass store straight to global memory, as the ragged kernel does, measured
// 0.5-2 % slower here: with one tile per CTA, other CTAs already cover the store phase.)
template <class T, bool FWD, class Lines>
__device__ __forceinline__ void process_tile(const GroupDesc& g, const Lines& lines, int64_t s0,
                                             int C, const typename Prec<T>::C* in,
                                             typename Prec<T>::C* out, typename Prec<T>::C* smem) {
  auto* A = smem;
  auto* B = smem + tile_elems(g.C, g.M);
  copy_tile<T, true>(A, in, nullptr, g, lines, s0, C);
  __syncthreads();
  // second group: the sub-problem index within the line enters the twiddle index
  const int64_t msub0 = g.twsub ? s0 : -1;
  A = run_passes<T, FWD>(g, A, B, C, msub0);
  copy_tile<T, false>(A, nullptr, out, g, lines, s0, C);
}

// binary64 names used by the FP64 kernels
template <bool FWD>
__device__ __forceinline__ double2* run_passes_f64(const GroupDesc& g, double2* A, double2* B,
                                                   int C, int64_t msub0) {
  return run_passes<double, FWD>(g, A, B, C, msub0);
}

template <bool FWD, class Lines>
__device__ __forceinline__ void process_tile_f64(const GroupDesc& g, const Lines& lines,
                                                 int64_t s0, int C, const double2* in,
                                                 double2* out, double2* smem) {
  process_tile<double, FWD>(g, lines, s0, C, in, out, smem);
}

}  // namespace dev
}  // namespace lfg
