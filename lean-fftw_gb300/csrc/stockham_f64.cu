// FP64 Stockham group kernel for sm_103a.
//
// One CTA loads a tile of C sub-problems of length M from global memory into shared memory
// (coalesced 16-byte complex loads), runs every pass of its group there with ping-pong
// buffers, and stores the tile back.  Each butterfly is a generated codelet
// (generated/codelets_f64.cuh) evaluated with explicitly rounded IEEE operations, so each
// pass performs exactly the operations of lean-fftw's reference pass
// (`LeanFFTW/Gen/Stockham.lean:263-284`); see stockham.h for why the grouping preserves this.
//
// On GB300 a binary64 FMA issues at about 2 lanes per clock per SM (1/64 of binary32), so
// this kernel is bound by the FP64 pipe, not by HBM: the codelets' operation counts, not
// memory traffic, set its speed.  Shared-memory layout and thread mapping only need to keep
// the FP64 pipe fed, which a few warps per SM do.
#include <cuda_runtime.h>

#include "generated/codelets_f64.cuh"
#include "kernels.h"
#include "stockham.h"

namespace lfg {
namespace {

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

// Copy a tile between global memory and a shared-memory tile buffer; the loop order makes
// consecutive threads touch consecutive global addresses (elements of a sub-problem when
// they are contiguous, else neighbouring sub-problems).
template <bool LOAD>
__device__ __forceinline__ void copy_tile(double2* tile, const double2* gin, double2* gout,
                                          const GroupDesc& g, int64_t s0, int C) {
  const int64_t line_st = LOAD ? g.in_line : g.out_line;
  const int64_t sub_st = LOAD ? g.in_sub : g.out_sub;
  const int64_t elem_st = LOAD ? g.in_elem : g.out_elem;
  const int M = g.M;
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
    const int64_t line = s / g.nsub;
    const int64_t sub = s - line * g.nsub;
    const int64_t a = line * line_st + sub * sub_st + (int64_t)i * elem_st;
    if (LOAD) tile[c * M + i] = gin[a];
    else gout[a] = tile[c * M + i];
  }
}

template <bool FWD>
__global__ void __launch_bounds__(kGroupThreads)
group_kernel_f64(const GroupDesc g, const double2* in, double2* out) {
  extern __shared__ double2 smem_f64[];
  const int64_t s0 = (int64_t)blockIdx.x * g.C;
  const int64_t rem = g.total_sub - s0;
  const int C = rem < g.C ? (int)rem : g.C;
  double2* A = smem_f64;
  double2* B = smem_f64 + (size_t)g.C * g.M;
  copy_tile<true>(A, in, nullptr, g, s0, C);
  __syncthreads();
  // second group: the sub-problem index within the line enters the twiddle index
  const int64_t msub0 = g.twsub ? (s0 % g.nsub) : -1;
  for (int t = 0; t < g.npass; ++t) {
    run_pass_f64<FWD>(A, B, C, g.M, g.pass[t], g.kmul, msub0);
    __syncthreads();
    double2* tmp = A;
    A = B;
    B = tmp;
  }
  copy_tile<false>(A, nullptr, out, g, s0, C);
}

}  // namespace

size_t group_smem_bytes_f64(const GroupDesc& g) { return 2 * (size_t)g.C * g.M * sizeof(double2); }

cudaError_t prepare_group_kernels_f64() {
  // the opt-in shared-memory limit is a property of the function in the current device's
  // context; the planner calls this once per plan, on the plan's device
  cudaError_t e = cudaFuncSetAttribute(group_kernel_f64<true>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)kMaxSmemBytes);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(group_kernel_f64<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)kMaxSmemBytes);
}

cudaError_t launch_group_f64(const GroupDesc& g, bool fwd, const void* in, void* out,
                             cudaStream_t stream) {
  const size_t smem = group_smem_bytes_f64(g);
  const int64_t grid = (g.total_sub + g.C - 1) / g.C;
  if (grid <= 0) return cudaSuccess;
  auto kern = fwd ? group_kernel_f64<true> : group_kernel_f64<false>;
  kern<<<(unsigned)grid, kGroupThreads, smem, stream>>>(g, static_cast<const double2*>(in),
                                                        static_cast<double2*>(out));
  return cudaGetLastError();
}

}  // namespace lfg
