// The instantiations of the persistent FP64 ragged kernel, one per (block shape, direction),
// each compiled in a translation unit of its own (ragged_f64.cu with -DLFG_PART=p).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "kernels.h"

namespace lfg {

using RaggedFn = void (*)(const RaggedClass*, const RaggedItem*, int, const int64_t*,
                          const int64_t*, const double2*, double2*, unsigned int*, double2*,
                          int64_t, int);

// Block shapes the autotuner chooses from: threads per CTA and the minimum resident CTAs per
// SM (which caps the registers per thread).
constexpr int ragged_shape_threads(int variant) {
  return variant == 1 ? 256 : variant == 2 ? 128 : variant == 3 ? 128 : variant == 4 ? 512 : 256;
}
constexpr int ragged_shape_min_blocks(int variant) {
  return variant == 1 ? 1 : variant == 2 ? 2 : variant == 3 ? 3 : variant == 4 ? 1 : 2;
}

// Part p = 2 * variant + (forward ? 1 : 0); defined in the part's own translation unit.
template <int P>
RaggedFn ragged_part_fn();
template <> RaggedFn ragged_part_fn<0>();
template <> RaggedFn ragged_part_fn<1>();
template <> RaggedFn ragged_part_fn<2>();
template <> RaggedFn ragged_part_fn<3>();
template <> RaggedFn ragged_part_fn<4>();
template <> RaggedFn ragged_part_fn<5>();
template <> RaggedFn ragged_part_fn<6>();
template <> RaggedFn ragged_part_fn<7>();
template <> RaggedFn ragged_part_fn<8>();
template <> RaggedFn ragged_part_fn<9>();
static_assert(kRaggedVariants == 5, "one part per (block shape, direction)");

}  // namespace lfg
