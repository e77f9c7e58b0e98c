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

#include <algorithm>

#include "ragged_parts.h"
#include "stockham_dev.cuh"

namespace lfg {
using namespace dev;
namespace {

template <bool FWD>
__global__ void __launch_bounds__(kGroupThreads)
group_kernel_f64(const GroupDesc g, const double2* in, double2* out) {
  extern __shared__ double2 smem_f64[];
  const int64_t s0 = (int64_t)blockIdx.x * g.C;
  const int64_t rem = g.total_sub - s0;
  const int C = rem < g.C ? (int)rem : g.C;
  process_tile_f64<FWD>(g, StridedLines{g.in_line, g.out_line}, s0, C, in, out, smem_f64);
}

}  // namespace

size_t group_smem_bytes_f64(const GroupDesc& g) {
  return 2 * (size_t)tile_elems(g.C, g.M) * sizeof(double2);
}

static RaggedFn ragged_fn(bool fwd, int variant) {
  switch (variant * 2 + (fwd ? 1 : 0)) {
    case 1: return ragged_part_fn<1>();
    case 2: return ragged_part_fn<2>();
    case 3: return ragged_part_fn<3>();
    case 4: return ragged_part_fn<4>();
    case 5: return ragged_part_fn<5>();
    case 6: return ragged_part_fn<6>();
    case 7: return ragged_part_fn<7>();
    case 8: return ragged_part_fn<8>();
    case 9: return ragged_part_fn<9>();
    default: return ragged_part_fn<0>();
  }
}

int ragged_variant_threads(int variant) { return ragged_shape_threads(variant); }

cudaError_t launch_ragged_f64(const RaggedLaunch& r, bool fwd, const void* in, void* out,
                              cudaStream_t stream, void* scratch, int64_t slab) {
  if (r.nitems <= 0) return cudaSuccess;
  RaggedFn kern = ragged_fn(fwd, r.variant);
  kern<<<r.grid, ragged_variant_threads(r.variant), r.smem, stream>>>(
      r.classes, r.items, r.nitems, r.in_off, r.out_off, static_cast<const double2*>(in),
      static_cast<double2*>(out), r.counter, static_cast<double2*>(scratch), slab, r.buf);
  return cudaGetLastError();
}

int ragged_blocks_per_sm_f64(size_t smem, int variant) {
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, ragged_fn(true, variant),
                                                    ragged_variant_threads(variant), smem) != cudaSuccess)
    return 1;
  return nb > 0 ? nb : 1;
}

// The opt-in shared-memory limit is a property of a function in the current device's
// context: allow each kernel the per-CTA maximum minus its static shared memory.  The planner
// calls this once per plan, on the plan's device.
template <class K>
cudaError_t allow_max_smem(K kern) {
  cudaFuncAttributes a;
  cudaError_t e = cudaFuncGetAttributes(&a, kern);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)(kMaxSmemBytes - a.sharedSizeBytes));
}

cudaError_t prepare_group_kernels_f64() {
  cudaError_t e;
  if ((e = allow_max_smem(group_kernel_f64<true>)) != cudaSuccess) return e;
  if ((e = allow_max_smem(group_kernel_f64<false>)) != cudaSuccess) return e;
  for (int v = 0; v < kRaggedVariants; ++v) {
    if ((e = allow_max_smem(ragged_fn(true, v))) != cudaSuccess) return e;
    if ((e = allow_max_smem(ragged_fn(false, v))) != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t launch_group_f64(const GroupDesc& gd, bool fwd, const void* in, void* out,
                             cudaStream_t stream) {
  GroupDesc g = gd;
  set_divisors(g);
  const size_t smem = group_smem_bytes_f64(g);
  const int64_t grid = (g.total_sub + g.C - 1) / g.C;
  if (grid <= 0) return cudaSuccess;
  auto kern = fwd ? group_kernel_f64<true> : group_kernel_f64<false>;
  kern<<<(unsigned)grid, kGroupThreads, smem, stream>>>(g, static_cast<const double2*>(in),
                                                        static_cast<double2*>(out));
  return cudaGetLastError();
}

}  // namespace lfg
