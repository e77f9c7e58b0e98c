// Persistent FP64 kernel over a ragged batch (one launch for all sizes).
//
// The kernel exists in kRaggedVariants block shapes and two directions; each of those ten
// instantiations carries the codelets of every radix three times over (one per tile
// source), so the build compiles this file once per instantiation, with -DLFG_PART=p
// (p = 2 * variant + (forward ? 1 : 0)), in parallel.  stockham_f64.cu gathers the parts.
#include <cuda_runtime.h>

#include "ragged_parts.h"
#include "stockham_dev.cuh"

#ifndef LFG_PART
#error "ragged_f64.cu is compiled once per part, with -DLFG_PART=0..9"
#endif

namespace lfg {
using namespace dev;
namespace {

// One fixed base per side (a single line): the two-group items that stage their
// intermediate in a CTA-private scratch slab instead of the output.
struct FixedBases {
  int64_t in_base, out_base;
  __device__ int64_t in(int64_t) const { return in_base; }
  __device__ int64_t out(int64_t) const { return out_base; }
  __device__ int64_t pitch(bool) const { return -1; }
};

// Each CTA takes work items from a queue (an atomic ticket counter, zeroed before the
// launch) until it is empty.  An item is a tile of up to C transforms of one size (one
// group), or one whole transform of a two-group size, whose first group writes its
// intermediate to the output and whose second group then works on the output in place; the
// barrier between them orders the global-memory traffic within the CTA.  Items are sorted
// by decreasing cost, so the largest start first.
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

constexpr int kVariant = LFG_PART / 2;
constexpr bool kFwd = (LFG_PART % 2) == 1;
static_assert(kVariant >= 0 && kVariant < kRaggedVariants, "LFG_PART out of range");

}  // namespace

template <>
RaggedFn ragged_part_fn<LFG_PART>() {
  return ragged_kernel_f64<kFwd, ragged_shape_threads(kVariant), ragged_shape_min_blocks(kVariant)>;
}

}  // namespace lfg
