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

// 16-byte asynchronous copy global -> shared (completion through cp.async groups).
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(
                   (unsigned)__cvta_generic_to_shared(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// Request the tile of a one-group item (w.count whole transforms of length g.M, each a
// contiguous line at its listed offset) into stage buffer X, in the padded tile layout.
__device__ __forceinline__ void stage_item(double2* X, const GroupDesc& g, const RaggedItem& w,
                                           const int64_t* __restrict__ in_off, const double2* in) {
  const int M = g.M;
  const int PM = sub_pitch(M);
  const int n = w.count * M;
  const FastDiv fdm = g.fd_m;
  for (int idx = threadIdx.x; idx < n; idx += blockDim.x) {
    const int c = fdiv(idx, fdm);
    const int i = idx - c * M;
    cp_async16(X + c * PM + spad(i), in + __ldg(in_off + w.first + c) + i);
  }
  cp_async_commit();
}

// Each CTA takes work items from a queue (an atomic ticket counter, zeroed before the
// launch) until it is empty, holding one ticket ahead.  An item is a tile of up to C
// transforms of one size (one group), or one whole transform of a two-group size.  Items
// are sorted by decreasing cost, so the largest start first.
//
// Shared memory holds three tile buffers X, Y, Z of `buf` elements.  A one-group item's
// tile arrives in X by asynchronous copies; its first pass reads X and writes Y, and as
// soon as that pass is done the next item's tile (if it is a one-group item) is requested
// into X, so the copies overlap the remaining passes (Y <-> Z) and the stores of the
// current item.  A two-group item runs its two groups from Y and Z with plain tile copies:
// the first group writes its intermediate to the output (or, when `scratch` is given, to
// this CTA's slab of device memory, as when the buffers are host memory) and the second
// group then works on it, the barrier between them ordering the global-memory traffic
// within the CTA.  No CTA waits on another.
template <bool FWD, int NT, int MINB>
__global__ void __launch_bounds__(NT, MINB)
ragged_kernel_f64(const RaggedClass* __restrict__ classes, const RaggedItem* __restrict__ items,
                  int nitems, const int64_t* __restrict__ in_off,
                  const int64_t* __restrict__ out_off, const double2* in, double2* out,
                  unsigned int* counter, double2* scratch, int64_t slab, int buf) {
  extern __shared__ double2 smem_f64[];
  __shared__ int s_next;
  double2* const X = smem_f64;
  double2* const Y = smem_f64 + buf;
  double2* const Z = Y + buf;
  if (threadIdx.x == 0) s_next = (int)atomicAdd(counter, 1u);
  __syncthreads();
  int it = s_next;
  bool staged = false;   // the current item's tile has been requested into X
  __syncthreads();       // every thread has read s_next before it is overwritten
  while (it < nitems) {
    // ticket of the next item: thread 0 publishes it only after the first pass, so the
    // atomic's round trip overlaps that pass instead of delaying the CTA
    unsigned ticket = 0;
    if (threadIdx.x == 0) ticket = atomicAdd(counter, 1u);
    const RaggedItem w = items[it];
    const RaggedClass& rc = classes[w.cls];
    int next;
    bool next_staged = false;
    if (rc.ngroups == 1) {
      const GroupDesc& g = rc.g[0];
      if (!staged) stage_item(X, g, w, in_off, in);
      cp_async_wait_all();
      __syncthreads();   // X complete for every thread
      run_pass_t<double, FWD>(X, Y, w.count, g.M, g.pass[0], -1, g.nsub, g.fd_nsub);
      if (threadIdx.x == 0) s_next = (int)ticket;
      __syncthreads();   // X consumed; s_next visible
      next = s_next;
      if (next < nitems) {
        const RaggedItem wn = items[next];
        const RaggedClass& rn = classes[wn.cls];
        if (rn.ngroups == 1) {
          stage_item(X, rn.g[0], wn, in_off, in);
          next_staged = true;
        }
      }
      double2* A = Y;
      double2* B = Z;
      for (int t = 1; t < g.npass; ++t) {
        run_pass_t<double, FWD>(A, B, w.count, g.M, g.pass[t], -1, g.nsub, g.fd_nsub);
        __syncthreads();
        double2* tmp = A;
        A = B;
        B = tmp;
      }
      copy_tile<double, false>(A, nullptr, out, g, ListedLines{in_off, out_off, w.first}, 0, w.count);
    } else {
      if (threadIdx.x == 0) s_next = (int)ticket;
      __syncthreads();   // s_next visible
      next = s_next;
      if (next < nitems) {
        const RaggedItem wn = items[next];
        const RaggedClass& rn = classes[wn.cls];
        if (rn.ngroups == 1) {   // X is idle during a two-group item
          stage_item(X, rn.g[0], wn, in_off, in);
          next_staged = true;
        }
      }
      const GroupDesc& g1 = rc.g[0];
      const GroupDesc& g2 = rc.g[1];
      if (scratch) {
        // intermediate in this CTA's slab of device memory (the output may be host memory)
        double2* mine = scratch + (int64_t)blockIdx.x * slab;
        const FixedBases first{__ldg(in_off + w.first), 0};
        const FixedBases second{0, __ldg(out_off + w.first)};
        for (int64_t s0 = 0; s0 < g1.nsub; s0 += g1.C) {
          process_tile_f64<FWD>(g1, first, s0, (int)min((int64_t)g1.C, g1.nsub - s0), in, mine, Y);
          __syncthreads();
        }
        for (int64_t s0 = 0; s0 < g2.nsub; s0 += g2.C) {
          process_tile_f64<FWD>(g2, second, s0, (int)min((int64_t)g2.C, g2.nsub - s0), mine, out, Y);
          __syncthreads();
        }
      } else {
        const ListedLines lines{in_off, out_off, w.first};
        for (int64_t s0 = 0; s0 < g1.nsub; s0 += g1.C) {
          process_tile_f64<FWD>(g1, lines, s0, (int)min((int64_t)g1.C, g1.nsub - s0), in, out, Y);
          __syncthreads();
        }
        // the second group reads the first group's result from the output
        const ListedLines inner{out_off, out_off, w.first};
        for (int64_t s0 = 0; s0 < g2.nsub; s0 += g2.C) {
          process_tile_f64<FWD>(g2, inner, s0, (int)min((int64_t)g2.C, g2.nsub - s0), out, out, Y);
          __syncthreads();
        }
      }
    }
    __syncthreads();   // buffers free for reuse; every thread has read s_next
    it = next;
    staged = next_staged;
  }
  cp_async_wait_all();   // (nothing is outstanding here: a staged item is always processed)
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
