// binary32 Stockham group kernel for sm_103a (the FP32 variant of the path).
//
// Same structure as the binary64 group kernel (stockham_f64.cu): one CTA loads a tile of
// sub-problems into shared memory, runs every pass of its group there, stores the tile.
// The butterflies are the same generated operation DAGs evaluated in binary32; twiddle tables
// are the binary64 exact-integer tables rounded to binary32, and the passes the planner marks
// (the last passes of sizes >= 2^16) multiply by twiddles held as binary32 (hi, lo) pairs with
// compensated products, which removes the twiddle-rounding error from those passes.  At 8
// bytes per point and 37 T binary32 instructions/s this variant is bound by HBM, not by the
// arithmetic.
#include <cuda_runtime.h>

#include "stockham_dev.cuh"

namespace lfg {
using namespace dev;
namespace {

template <bool FWD>
__global__ void __launch_bounds__(kGroupThreads)
group_kernel_f32(const GroupDesc g, const float2* in, float2* out) {
  extern __shared__ float2 smem_f32[];
  const int64_t s0 = (int64_t)blockIdx.x * g.C;
  const int64_t rem = g.total_sub - s0;
  const int C = rem < g.C ? (int)rem : g.C;
  process_tile<float, FWD>(g, StridedLines{g.in_line, g.out_line}, s0, C, in, out, smem_f32);
}

template <class K>
cudaError_t allow_max_smem(K kern) {
  cudaFuncAttributes a;
  cudaError_t e = cudaFuncGetAttributes(&a, kern);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)(kMaxSmemBytes - a.sharedSizeBytes));
}

}  // namespace

cudaError_t prepare_group_kernels_f32() {
  cudaError_t e = allow_max_smem(group_kernel_f32<true>);
  if (e != cudaSuccess) return e;
  return allow_max_smem(group_kernel_f32<false>);
}

cudaError_t launch_group_f32(const GroupDesc& g, bool fwd, const void* in, void* out,
                             cudaStream_t stream) {
  const size_t smem = 2 * (size_t)g.C * g.M * sizeof(float2);
  const int64_t grid = (g.total_sub + g.C - 1) / g.C;
  if (grid <= 0) return cudaSuccess;
  auto kern = fwd ? group_kernel_f32<true> : group_kernel_f32<false>;
  kern<<<(unsigned)grid, kGroupThreads, smem, stream>>>(g, static_cast<const float2*>(in),
                                                        static_cast<float2*>(out));
  return cudaGetLastError();
}

}  // namespace lfg
