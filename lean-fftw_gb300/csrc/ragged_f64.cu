// Persistent FP64 kernel over a ragged batch (one launch for all sizes).
//
// The kernel exists in kRaggedVariants block shapes and two directions; each of those ten
// instantiations carries the codelets of every radix three times over (one per pass
// destination: shared memory, or the output rows of a line list or of a scratch slab), so
// the build compiles this file once per instantiation, with -DLFG_PART=p
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

// 16-byte asynchronous copy global -> shared (completion through cp.async groups).  The
// L1-allocating form (.ca): when the source is pinned host memory read over NVLink-C2C, the
// L2-only form (.cg) made the whole 8192-size batch 45 % slower end to end (3.24 against
// 2.24 ms); on device memory the two are within 1 %.
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 16;" ::"r"(
                   (unsigned)__cvta_generic_to_shared(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// Request a tile of C sub-problems of group g, starting at sub-problem s0, from `src` into
// stage buffer X (padded tile layout), with the element order of copy_tile's loads:
// consecutive threads take consecutive elements of a sub-problem when those are contiguous
// (in_elem == 1), else neighbouring sub-problems.  Each thread walks its elements with
// running (sub-problem, element) indices -- one division per tile, not three per element --
// and a tile inside one line (every tile of a two-group item) reads that line's base once.
// The copies are spread over threads tid = 0 .. S-1 of the calling subset (all the CTA's
// threads, or the warps without work in the pass that runs meanwhile).
template <class Lines>
__device__ __forceinline__ void stage_tile(double2* X, const GroupDesc& g, const Lines& lines,
                                           int64_t s0, int C, const double2* src, int tid, int S) {
  // descriptor fields in registers: each cp.async below is a compiler memory barrier, after
  // which fields read through a reference would be loaded again for every element
  const int64_t sub_st = g.in_sub, elem_st = g.in_elem;
  const int M = g.M;
  const int nsub = g.nsub;
  const int gC = g.C;
  const FastDiv fd_m = g.fd_m, fd_c = g.fd_c, fd_nsub = g.fd_nsub;
  const Lines L = lines;
  const bool elem_fast = elem_st == 1;
  const int64_t line0 = s0 / nsub;
  const int sub0 = (int)(s0 - line0 * nsub);
  const int PM = sub_pitch(M);
  if (elem_fast) {
    // idx = c * M + i over the C sub-problems present
    const int nn = C * M;
    int c = fdiv(tid, fd_m);
    int i = tid - c * M;
    const int dc = fdiv(S, fd_m), di = S - dc * M;
    for (int idx = tid; idx < nn; idx += S) {
      const int t = sub0 + c;
      const int ql = fdiv(t, fd_nsub);
      const int64_t a = L.in(line0 + ql) + (int64_t)(t - ql * nsub) * sub_st + i;
      cp_async16(X + c * PM + spad(i), src + a);
      c += dc;
      i += di;
      if (i >= M) {
        i -= M;
        ++c;
      }
    }
  } else {
    // idx = i * gC + c over the full tile width (a partial tile skips the missing columns)
    const int nn = gC * M;
    int i = fdiv(tid, fd_c);
    int c = tid - i * gC;
    const int di = fdiv(S, fd_c), dc = S - di * gC;
    if (sub0 + C <= nsub) {
      // one line: its base once, then (sub0 + c) * sub_st + i * elem_st
      const double2* base = src + L.in(line0) + (int64_t)sub0 * sub_st;
      for (int idx = tid; idx < nn; idx += S) {
        if (c < C) cp_async16(X + c * PM + spad(i), base + (int64_t)c * sub_st + (int64_t)i * elem_st);
        c += dc;
        i += di;
        if (c >= gC) {
          c -= gC;
          ++i;
        }
      }
    } else {
      for (int idx = tid; idx < nn; idx += S) {
        if (c < C) {
          const int t = sub0 + c;
          const int ql = fdiv(t, fd_nsub);
          const int64_t a = L.in(line0 + ql) + (int64_t)(t - ql * nsub) * sub_st + (int64_t)i * elem_st;
          cp_async16(X + c * PM + spad(i), src + a);
        }
        c += dc;
        i += di;
        if (c >= gC) {
          c -= gC;
          ++i;
        }
      }
    }
  }
  cp_async_commit();
}

// One tile of an item: its group, first sub-problem and number of sub-problems.  A one-group
// item is one task; a two-group item is the tiles of its first group, then those of its
// second group.
struct Task {
  int grp;
  int C;
  int64_t s0;
};

__device__ __forceinline__ int first_group_tasks(const RaggedClass& rc) {
  return (rc.g[0].nsub + rc.g[0].C - 1) / rc.g[0].C;
}
__device__ __forceinline__ int task_count(const RaggedClass& rc) {
  return rc.ngroups == 1 ? 1 : first_group_tasks(rc) + (rc.g[1].nsub + rc.g[1].C - 1) / rc.g[1].C;
}
__device__ __forceinline__ Task task_of(const RaggedClass& rc, const RaggedItem& w, int k) {
  if (rc.ngroups == 1) return Task{0, w.count, 0};
  const int n1 = first_group_tasks(rc);
  const int grp = k < n1 ? 0 : 1;
  const GroupDesc& g = rc.g[grp];
  const int64_t s0 = (int64_t)(grp == 0 ? k : k - n1) * g.C;
  return Task{grp, (int)min((int64_t)g.C, (int64_t)g.nsub - s0), s0};
}

// Where a task's tile comes from and goes to.  One group: listed lines, in -> out.  Two
// groups: the first group reads the input line and writes the intermediate, the second reads
// the intermediate and writes the output line; the intermediate is the output line itself, or
// this CTA's slab `mine` of device memory when one is given (the buffers may be host memory).
struct TaskIO {
  const int64_t* __restrict__ in_off;
  const int64_t* __restrict__ out_off;
  const double2* in;
  double2* out;
  double2* mine;

  __device__ __forceinline__ void stage(double2* X, const RaggedClass& rc, const RaggedItem& w,
                                        const Task& t, int tid, int S) const {
    const GroupDesc& g = rc.g[t.grp];
    if (rc.ngroups == 1 || (!mine && t.grp == 0)) {
      stage_tile(X, g, ListedLines{in_off, out_off, w.first}, t.s0, t.C, in, tid, S);
    } else if (!mine) {
      stage_tile(X, g, ListedLines{out_off, out_off, w.first}, t.s0, t.C, out, tid, S);
    } else if (t.grp == 0) {
      stage_tile(X, g, FixedBases{__ldg(in_off + w.first), 0}, t.s0, t.C, in, tid, S);
    } else {
      stage_tile(X, g, FixedBases{0, 0}, t.s0, t.C, mine, tid, S);
    }
  }

  // Tasks whose outputs are contiguous runs per sub-problem (one-group items, first groups)
  // let their last pass store straight to global memory: consecutive threads write
  // consecutive elements of a run, and the tile's round trip through shared memory, with
  // its barrier, disappears.
  __device__ __forceinline__ bool direct(const RaggedClass& rc, const Task& t) const {
    const GroupDesc& g = rc.g[t.grp];
    return (rc.ngroups == 1 || t.grp == 0) && g.out_elem == 1 && g.unit_scale;
  }

  template <bool FWD>
  __device__ __forceinline__ void last_pass(const double2* A, const RaggedClass& rc,
                                            const RaggedItem& w, const Task& t, const PassDesc& pd,
                                            int sub0) const {
    const GroupDesc& g = rc.g[t.grp];
    if (mine && rc.ngroups == 2) {
      run_pass_to<double, FWD>(A, GlobalRows<double, FixedBases>{mine, g, FixedBases{0, 0}, 0, (int)t.s0},
                               t.C, g.M, pd, sub0, g.nsub, g.fd_nsub);
    } else {
      run_pass_to<double, FWD>(A, GlobalRows<double, ListedLines>{out, g, ListedLines{in_off, out_off, w.first},
                                                                  0, (int)t.s0},
                               t.C, g.M, pd, sub0, g.nsub, g.fd_nsub);
    }
  }

  __device__ __forceinline__ void store(double2* A, const RaggedClass& rc, const RaggedItem& w,
                                        const Task& t) const {
    const GroupDesc& g = rc.g[t.grp];
    if (rc.ngroups == 1 || (!mine && t.grp == 0)) {
      copy_tile<double, false>(A, nullptr, out, g, ListedLines{in_off, out_off, w.first}, t.s0, t.C);
    } else if (!mine) {
      copy_tile<double, false>(A, nullptr, out, g, ListedLines{out_off, out_off, w.first}, t.s0, t.C);
    } else if (t.grp == 0) {
      copy_tile<double, false>(A, nullptr, mine, g, FixedBases{0, 0}, t.s0, t.C);
    } else {
      copy_tile<double, false>(A, nullptr, out, g, FixedBases{0, __ldg(out_off + w.first)}, t.s0, t.C);
    }
  }
};

// Each CTA takes work items from a queue (an atomic ticket counter, zeroed before the
// launch) until it is empty, holding one ticket ahead.  An item is a tile of up to C
// transforms of one size (one group), or one whole transform of a two-group size.  Items
// are sorted by decreasing cost, so the largest start first.
//
// Shared memory holds three tile buffers X, Y, Z of `buf` elements.  Every task's tile
// arrives in X by asynchronous copies; its first pass reads X and writes Y, and as soon as
// that pass is done the next task's tile is requested into X (the next tile of this item,
// or the first tile of the next item), so the copies overlap the remaining passes (Y <-> Z)
// and the stores of the current task.  The one tile not requested ahead is the first of a
// second group: it reads what the last tile of the first group stores, so it is requested
// after the barrier that ends that task (a barrier orders a CTA's global-memory accesses).
// No CTA waits on another.
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
  const TaskIO io{in_off, out_off, in, out, scratch ? scratch + (int64_t)blockIdx.x * slab : nullptr};
  if (threadIdx.x == 0) s_next = (int)atomicAdd(counter, 1u);
  __syncthreads();
  int it = s_next;
  bool staged = false;   // the current task's tile has been requested into X
  __syncthreads();       // every thread has read s_next before it is overwritten
  while (it < nitems) {
    // ticket of the next item: thread 0 publishes it only after the first pass, so the
    // atomic's round trip overlaps that pass instead of delaying the CTA
    unsigned ticket = 0;
    if (threadIdx.x == 0) ticket = atomicAdd(counter, 1u);
    const RaggedItem w = items[it];
    const RaggedClass& rc = classes[w.cls];
    const int nt = task_count(rc);
    int next = nitems;
    for (int k = 0; k < nt; ++k) {
      const Task t = task_of(rc, w, k);
      const GroupDesc& g = rc.g[t.grp];
      if (!staged) io.stage(X, rc, w, t, threadIdx.x, NT);
      cp_async_wait_all();
      __syncthreads();   // X complete for every thread
      const int sub0 = g.twsub ? (int)(t.s0 % g.nsub) : -1;
      const bool direct = io.direct(rc, t);
      const int np = g.npass;
      if (np == 1 && direct) io.template last_pass<FWD>(X, rc, w, t, g.pass[0], sub0);
      else run_pass_t<double, FWD>(X, Y, t.C, g.M, g.pass[0], sub0, g.nsub, g.fd_nsub);
      if (k == 0 && threadIdx.x == 0) s_next = (int)ticket;
      __syncthreads();   // X consumed; s_next visible
      if (k == 0) next = s_next;
      staged = false;
      // who requests the next tile: when the next pass leaves two or more warps without a
      // butterfly, those warps do, while the others run the pass (the copies' address
      // arithmetic then overlaps the FP64 work); otherwise every thread, before the pass
      int s_tid = threadIdx.x, s_n = NT;
      if (np > 1) {
        const int busy = ((t.C * (g.M / g.pass[1].R) + 31) / 32) * 32;
        if (busy <= NT - 64) {
          s_tid = (int)threadIdx.x - busy;
          s_n = NT - busy;
        }
      }
      if (k + 1 < nt) {
        const Task tn = task_of(rc, w, k + 1);
        if (tn.grp == t.grp) {
          if (s_tid >= 0) io.stage(X, rc, w, tn, s_tid, s_n);
          staged = true;
        }
      } else if (next < nitems) {
        if (s_tid >= 0) {
          const RaggedItem wn = items[next];
          const RaggedClass& rn = classes[wn.cls];
          io.stage(X, rn, wn, task_of(rn, wn, 0), s_tid, s_n);
        }
        staged = true;
      }
      double2* A = Y;
      double2* B = Z;
      for (int p = 1; p < np; ++p) {
        if (p == np - 1 && direct) {
          io.template last_pass<FWD>(A, rc, w, t, g.pass[p], sub0);
          break;
        }
        run_pass_t<double, FWD>(A, B, t.C, g.M, g.pass[p], sub0, g.nsub, g.fd_nsub);
        __syncthreads();
        double2* tmp = A;
        A = B;
        B = tmp;
      }
      if (!direct) io.store(A, rc, w, t);
      __syncthreads();   // buffers free for reuse; this task's stores ordered before later loads
    }
    it = next;
  }
  cp_async_wait_all();   // (nothing is outstanding here: a requested tile is always processed)
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
