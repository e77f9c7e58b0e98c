// Device-side building blocks of the FP64 Stockham kernels (pass, tile copy, tile driver).
//
// Each butterfly is a generated codelet (generated/codelets_f64.cuh) evaluated with
// explicitly rounded IEEE operations, so each pass performs exactly the operations of
// lean-fftw's reference pass (`LeanFFTW/Gen/Stockham.lean:263-284`); stockham.h explains why
// grouping passes over sub-problems preserves this.
#pragma once
#include <cuda_runtime.h>

#include "generated/codelets_f64.cuh"
#include "kernels.h"
#include "stockham.h"

namespace lfg {
namespace dev {


// One pass over the C sub-problems of a tile: src, dst are tile buffers in shared memory.
template <bool FWD, int R, bool TW>
__device__ __forceinline__ void pass_f64(const double2* __restrict__ src, double2* __restrict__ dst,
                                         int C, int M, const PassDesc& pd, int kmul, int64_t msub0) {
  const int MR = M / R;
  const int nb = C * MR;
  const int ns = pd.ns_loc;
  const double* __restrict__ tw = static_cast<const double*>(pd.tw);
  const int64_t nsg = pd.ns_g;
  for (int q = threadIdx.x; q < nb; q += blockDim.x) {
    const int c = q / MR;
    const int j = q - c * MR;
    double x[TW ? 4 * R - 2 : 2 * R];
    double y[2 * R];
    const double2* s = src + c * M + j;
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const double2 v = s[r * MR];
      x[2 * r] = v.x;
      x[2 * r + 1] = v.y;
    }
    const int k = j % ns;
    if (TW) {
      // table index of the twiddle: k_loc * kmul + sub-problem index (second group only)
      const int64_t kg = (int64_t)k * kmul + (msub0 >= 0 ? msub0 + c : 0);
#pragma unroll
      for (int r = 0; r < R - 1; ++r) {
        x[2 * R + 2 * r] = __ldg(tw + 2 * r * nsg + kg);
        x[2 * R + 2 * r + 1] = __ldg(tw + (2 * r + 1) * nsg + kg);
      }
    }
    BflyD<FWD, R, TW>::run(x, y);
    const int b = j / ns;
    double2* d = dst + c * M + b * ns * R + k;
#pragma unroll
    for (int r = 0; r < R; ++r) d[r * ns] = make_double2(y[2 * r], y[2 * r + 1]);
  }
}

template <bool FWD>
__device__ __forceinline__ void run_pass_f64(const double2* src, double2* dst, int C, int M,
                                             const PassDesc& pd, int kmul, int64_t msub0) {
#define LFG_PASS_CASE(RR)                                                   \
  case RR:                                                                  \
    if (pd.tw) pass_f64<FWD, RR, true>(src, dst, C, M, pd, kmul, msub0);    \
    else pass_f64<FWD, RR, false>(src, dst, C, M, pd, kmul, msub0);         \
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

// Line bases (complex-element offsets of each line) of the two tile sources: evenly strided
// lines of a batched plan, or a list of per-transform offsets of a ragged batch.
struct StridedLines {
  int64_t in_line, out_line;
  __device__ int64_t in(int64_t line) const { return line * in_line; }
  __device__ int64_t out(int64_t line) const { return line * out_line; }
};

struct ListedLines {
  const int64_t* __restrict__ in_off;
  const int64_t* __restrict__ out_off;
  int64_t first;
  __device__ int64_t in(int64_t line) const { return __ldg(in_off + first + line); }
  __device__ int64_t out(int64_t line) const { return __ldg(out_off + first + line); }
};

// Copy a tile between global memory and a shared-memory tile buffer; the loop order makes
// consecutive threads touch consecutive global addresses (elements of a sub-problem when
// they are contiguous, else neighbouring sub-problems).
template <bool LOAD, class Lines>
__device__ __forceinline__ void copy_tile(double2* tile, const double2* gin, double2* gout,
                                          const GroupDesc& g, const Lines& lines, int64_t s0,
                                          int C) {
  const int64_t sub_st = LOAD ? g.in_sub : g.out_sub;
  const int64_t elem_st = LOAD ? g.in_elem : g.out_elem;
  const int M = g.M;
  const int nsub = g.nsub;
  const int n = C * M;
  const bool elem_fast = (elem_st == 1);
  for (int idx = threadIdx.x; idx < n; idx += blockDim.x) {
    int c, i;
    if (elem_fast) {
      c = idx / M;
      i = idx - c * M;
    } else {
      i = idx / C;
      c = idx - i * C;
    }
    const int64_t s = s0 + c;
    const int64_t line = s / nsub;
    const int64_t sub = s - line * nsub;
    const int64_t a = (LOAD ? lines.in(line) : lines.out(line)) + sub * sub_st + (int64_t)i * elem_st;
    if (LOAD) {
      tile[c * M + i] = gin[a];
    } else if (g.scale == 1.0) {
      gout[a] = tile[c * M + i];
    } else {
      const double2 v = tile[c * M + i];
      gout[a] = make_double2(__dmul_rn(v.x, g.scale), __dmul_rn(v.y, g.scale));
    }
  }
}

// Run every pass of group g on a tile of C sub-problems held in shared-memory buffer A
// (B is the ping-pong partner); returns the buffer holding the result.
template <bool FWD>
__device__ __forceinline__ double2* run_passes_f64(const GroupDesc& g, double2* A, double2* B,
                                                   int C, int64_t msub0) {
  const int npass = g.npass;
  for (int t = 0; t < npass; ++t) {
    run_pass_f64<FWD>(A, B, C, g.M, g.pass[t], g.kmul, msub0);
    __syncthreads();
    double2* tmp = A;
    A = B;
    B = tmp;
  }
  return A;
}

// Load C sub-problems starting at s0, run every pass of group g in shared memory, store.
template <bool FWD, class Lines>
__device__ __forceinline__ void process_tile_f64(const GroupDesc& g, const Lines& lines,
                                                 int64_t s0, int C, const double2* in,
                                                 double2* out, double2* smem) {
  double2* A = smem;
  double2* B = smem + (size_t)g.C * g.M;
  copy_tile<true>(A, in, nullptr, g, lines, s0, C);
  __syncthreads();
  // second group: the sub-problem index within the line enters the twiddle index
  const int64_t msub0 = g.twsub ? (s0 % g.nsub) : -1;
  const int npass = g.npass;
  for (int t = 0; t < npass; ++t) {
    run_pass_f64<FWD>(A, B, C, g.M, g.pass[t], g.kmul, msub0);
    __syncthreads();
    double2* tmp = A;
    A = B;
    B = tmp;
  }
  copy_tile<false>(A, nullptr, out, g, lines, s0, C);
}

}  // namespace dev
}  // namespace lfg
