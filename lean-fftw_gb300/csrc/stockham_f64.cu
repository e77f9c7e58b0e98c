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

// Persistent kernel over a ragged batch: each CTA takes work items from a queue (an atomic
// ticket counter, zeroed before the launch) until it is empty.  An item is a tile of up to
// C transforms of one size (one group), or one whole transform of a two-group size, whose
// first group writes its intermediate to the output and whose second group then works on
// the output in place; the barrier between them orders the global-memory traffic within
// the CTA.  Items are sorted by decreasing cost, so the largest start first.
// One fixed base per side (a single line): the two-group items that stage their
// intermediate in a CTA-private scratch slab instead of the output.
struct FixedBases {
  int64_t in_base, out_base;
  __device__ int64_t in(int64_t) const { return in_base; }
  __device__ int64_t out(int64_t) const { return out_base; }
  __device__ int64_t pitch(bool) const { return -1; }
};

template <bool FWD, int NT, int MINB>
__global__ void __launch_bounds__(NT, MINB)
ragged_kernel_f64(const RaggedClass* __restrict__ classes, const RaggedItem* __restrict__ items,
                  int nitems, const int64_t* __restrict__ in_off,
                  const int64_t* __restrict__ out_off, const double2* in, double2* out,
                  unsigned int* counter, double2* scratch, int64_t slab) {
  extern __shared__ double2 smem_f64[];
  __shared__ int s_item;
  for (;;) {
    if (threadIdx.x == 0) s_item = (int)atomicAdd(counter, 1u);
    __syncthreads();
    const int it = s_item;
    if (it >= nitems) break;
    const RaggedItem w = items[it];
    const RaggedClass& rc = classes[w.cls];
    const ListedLines lines{in_off, out_off, w.first};
    if (rc.ngroups == 1) {
      process_tile_f64<FWD>(rc.g[0], lines, 0, w.count, in, out, smem_f64);
    } else if (scratch) {
      // intermediate in this CTA's slab of device memory (the output may be host memory)
      const GroupDesc& g1 = rc.g[0];
      const GroupDesc& g2 = rc.g[1];
      double2* mine = scratch + (int64_t)blockIdx.x * slab;
      const FixedBases first{__ldg(in_off + w.first), 0};
      const FixedBases second{0, __ldg(out_off + w.first)};
      for (int64_t s0 = 0; s0 < g1.nsub; s0 += g1.C) {
        process_tile_f64<FWD>(g1, first, s0, (int)min((int64_t)g1.C, g1.nsub - s0), in, mine, smem_f64);
        __syncthreads();
      }
      for (int64_t s0 = 0; s0 < g2.nsub; s0 += g2.C) {
        process_tile_f64<FWD>(g2, second, s0, (int)min((int64_t)g2.C, g2.nsub - s0), mine, out, smem_f64);
        __syncthreads();
      }
    } else {
      const GroupDesc& g1 = rc.g[0];
      const GroupDesc& g2 = rc.g[1];
      for (int64_t s0 = 0; s0 < g1.nsub; s0 += g1.C) {
        process_tile_f64<FWD>(g1, lines, s0, (int)min((int64_t)g1.C, g1.nsub - s0), in, out, smem_f64);
        __syncthreads();
      }
      // the second group reads the first group's result from the output
      const ListedLines inner{out_off, out_off, w.first};
      for (int64_t s0 = 0; s0 < g2.nsub; s0 += g2.C) {
        process_tile_f64<FWD>(g2, inner, s0, (int)min((int64_t)g2.C, g2.nsub - s0), out, out, smem_f64);
        __syncthreads();
      }
    }
    __syncthreads();   // every thread has read s_item before it is overwritten
  }
}

}  // namespace

size_t group_smem_bytes_f64(const GroupDesc& g) {
  return 2 * (size_t)tile_elems(g.C, g.M) * sizeof(double2);
}

size_t ragged_smem_bytes_f64(const RaggedClass& c) {
  size_t m = 0;
  for (int i = 0; i < c.ngroups; ++i) m = std::max(m, group_smem_bytes_f64(c.g[i]));
  return m;
}

// Block shapes of the persistent kernel the autotuner chooses from: (threads, minimum
// resident CTAs per SM, which caps the registers per thread).
using RaggedFn = void (*)(const RaggedClass*, const RaggedItem*, int, const int64_t*,
                          const int64_t*, const double2*, double2*, unsigned int*, double2*,
                          int64_t);

template <bool FWD>
RaggedFn ragged_fn(int variant) {
  switch (variant) {
    case 1: return ragged_kernel_f64<FWD, 256, 1>;
    case 2: return ragged_kernel_f64<FWD, 128, 2>;
    case 3: return ragged_kernel_f64<FWD, 128, 3>;
    case 4: return ragged_kernel_f64<FWD, 512, 1>;
    default: return ragged_kernel_f64<FWD, 256, 2>;
  }
}

int ragged_variant_threads(int variant) {
  switch (variant) {
    case 1: return 256;
    case 2: return 128;
    case 3: return 128;
    case 4: return 512;
    default: return 256;
  }
}

cudaError_t launch_ragged_f64(const RaggedLaunch& r, bool fwd, const void* in, void* out,
                              cudaStream_t stream, void* scratch, int64_t slab) {
  if (r.nitems <= 0) return cudaSuccess;
  RaggedFn kern = fwd ? ragged_fn<true>(r.variant) : ragged_fn<false>(r.variant);
  kern<<<r.grid, ragged_variant_threads(r.variant), r.smem, stream>>>(
      r.classes, r.items, r.nitems, r.in_off, r.out_off, static_cast<const double2*>(in),
      static_cast<double2*>(out), r.counter, static_cast<double2*>(scratch), slab);
  return cudaGetLastError();
}

int ragged_blocks_per_sm_f64(size_t smem, int variant) {
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, ragged_fn<true>(variant),
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
    if ((e = allow_max_smem(ragged_fn<true>(v))) != cudaSuccess) return e;
    if ((e = allow_max_smem(ragged_fn<false>(v))) != cudaSuccess) return e;
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
