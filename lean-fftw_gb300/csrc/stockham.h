// Descriptors shared by the host planner and the Stockham group kernels.
//
// A transform of size N = R_0 ... R_{s-1} runs s Stockham passes (lean-fftw
// `LeanFFTW/Gen/Stockham.lean:276-294`): pass t has ns = R_0 ... R_{t-1}; butterfly
// j = b*ns + k reads z[j + r*N/R], multiplies input r >= 1 by the table twiddle w_r(k) when
// t >= 1, and writes output r to position b*ns*R + k + r*ns.
//
// The GPU runs the passes in one or more *groups*.  A group is a run of consecutive passes
// whose data dependencies close over independent sub-problems of length M (the product of
// the group's radices), so one CTA can load a tile of sub-problems into shared memory, run
// every pass of the group there, and store the tile back:
//
//   * one group (N fits in shared memory): sub-problem = one whole transform;
//   * first of two groups (passes 0..T-1, product P): sub-problem b < N/P is the
//     stride-N/P subsequence x[b + (N/P) i], written contiguously to z[b*P + m];
//   * second group (passes T..s-1): sub-problem m < P is the stride-P subsequence
//     z[q*P + m]; it is read and written in place, and the table index of a twiddle is
//     k = k_local*P + m (for the shared-memory group kernels the planner stores these tables
//     transposed, at m*ns_local + k_local, so that a warp's threads, which walk k_local, read
//     neighbouring entries; the binary32 register-staged kernels walk m and keep pass order).
//
// Both facts follow from the pass formula: after passes 0..T-1, positions b*P..b*P+P-1 hold
// the size-P transform of x[b + (N/P) i]; every later pass maps positions = m (mod P) to
// positions = m (mod P), since N/R and ns are multiples of P.  Each butterfly therefore
// performs exactly the operations of the reference pass, so the result is bit-identical to
// the reference transform for the same radix sequence.
#pragma once
#include <cstdint>

#ifdef __CUDACC__
#define LFG_HD __host__ __device__
#else
#define LFG_HD
#endif

namespace lfg {

constexpr int kMaxPass = 24;       // lean-fftw Asm/Planner.lean:49 (`maxPass`)
constexpr int kMaxRadix = 16;

// Division of 0 <= n < 2^31 by a divisor d >= 1 fixed at plan time, as one multiply-high, an
// add and a shift: q = (umulhi(m, n) + n) >> l with l = ceil(log2 d) and
// m = floor(2^32 (2^l - d) / d) + 1 (Granlund and Montgomery, "Division by invariant integers
// using multiplication", PLDI 1994, Fig. 4.1, specialised to 31-bit dividends so that the sum
// cannot overflow).  The kernels' index arithmetic divides by sub-problem lengths, tile sizes
// and pass strides that only the plan knows.
struct FastDiv {
  uint32_t m;
  uint32_t l;
};

inline FastDiv make_fastdiv(int d) {
  uint32_t l = 0;
  while (l < 31 && (1u << l) < (uint32_t)d) ++l;
  const uint64_t m = ((uint64_t(1) << 32) * ((uint64_t(1) << l) - (uint64_t)d)) / (uint64_t)d + 1;
  return FastDiv{(uint32_t)m, l};
}

// Host-side evaluation of the same formula (tests, planner checks).
inline int fastdiv_host(int n, FastDiv f) {
  const uint32_t t = (uint32_t)(((uint64_t)f.m * (uint32_t)n) >> 32);
  return (int)((t + (uint32_t)n) >> f.l);
}

// Shared-memory tile layout: sub-problem c of a tile starts at c * sub_pitch(M), and its
// element i sits at i + i/16 (one padding element after every 16).  The padding spreads a
// pass's stride-R stores over the banks.  Across sub-problems: a warp of a pass whose
// sub-problems hold few butterflies spans several sub-problems at element stride 17, which
// the pitch M + M/16 (= 17 M/16) keeps conflict-free for M a multiple of 16; for other M an
// odd pitch puts neighbouring sub-problems in different banks.  (An odd pitch for large
// multiples of 16 removes the conflicts of strided tile copies too, but measured slower on
// the binary32 stream kernel and no faster elsewhere.)
LFG_HD constexpr int sub_pitch(int M) {
  return (M & 15) == 0 ? M + (M >> 4) : (M + (M >> 4)) | 1;
}
LFG_HD constexpr int64_t tile_elems(int64_t C, int M) { return C * (int64_t)sub_pitch(M); }

struct PassDesc {
  int R;                 // radix of the pass
  int ns_loc;            // product of the group's earlier radices
  int ns_g;              // product of all earlier radices of the transform (table row length)
  int comp;              // binary32 only: twiddles as (hi, lo) pairs, compensated products
  const void* tw;        // pass twiddle table (2*(R-1)*ns_g scalars; binary32 comp passes:
                         // the hi table followed by the lo table), nullptr for pass 0
  FastDiv fd_mr;         // divisor M / R (butterflies per sub-problem)
  FastDiv fd_ns;         // divisor ns_loc
};

// Complex element (s, i) of sub-problem s (flattened over lines) lives at
//   base + (s / nsub) * line_stride + (s % nsub) * sub_stride + i * elem_stride
// in units of complex elements, separately for input and output.
struct GroupDesc {
  int M;                 // sub-problem length
  int npass;
  int nsub;              // sub-problems per line
  int C;                 // sub-problems per CTA tile
  int64_t total_sub;     // lines * nsub
  int64_t in_line, in_sub, in_elem;
  int64_t out_line, out_sub, out_elem;
  int kmul;              // product of the radices before the group (P for a second group)
  int twsub;
  double scale;          // outputs multiplied by this on store unless it is exactly 1
  int unit_scale;        // scale == 1 (set_divisors: kernels test it without an FP64 compare)
  float scale_f32;       // scale rounded to binary32 (set_divisors)
  FastDiv fd_m, fd_c, fd_nsub;   // divisors M, C, nsub (set_divisors)
  PassDesc pass[kMaxPass];
};

// Fill the FastDiv fields from M, C, nsub and the passes; every launch path calls this on
// the descriptor it passes to a kernel, so planners may change C freely before.
inline void set_divisors(GroupDesc& g) {
  g.unit_scale = g.scale == 1.0 ? 1 : 0;
  g.scale_f32 = (float)g.scale;
  g.fd_m = make_fastdiv(g.M > 0 ? g.M : 1);
  g.fd_c = make_fastdiv(g.C > 0 ? g.C : 1);
  g.fd_nsub = make_fastdiv(g.nsub > 0 ? g.nsub : 1);
  for (int t = 0; t < g.npass && t < kMaxPass; ++t) {
    PassDesc& d = g.pass[t];
    d.fd_mr = make_fastdiv(d.R > 0 ? g.M / d.R : 1);
    d.fd_ns = make_fastdiv(d.ns_loc > 0 ? d.ns_loc : 1);
  }
}

// One distinct size of a ragged batch: one group, or two groups run back to back by one CTA
// (first group to the output, second group in place on the output).  Line strides of the
// GroupDescs are unused; lines are located through per-transform offsets.
struct RaggedClass {
  GroupDesc g[2];
  int ngroups;
  int n;
};

// A work item: `count` transforms of class `cls`, the lines first .. first+count-1 of the
// offset lists (sorted by class).
struct RaggedItem {
  int cls;
  int count;
  int64_t first;
};

struct RaggedLaunch {
  const RaggedClass* classes;
  const RaggedItem* items;
  int nitems;
  const int64_t* in_off;
  const int64_t* out_off;
  unsigned int* counter;
  unsigned grid;
  size_t smem;           // three tile buffers of `buf` complex elements
  int buf;
  int variant;           // block shape of the persistent kernel (kernels.h)
};

}  // namespace lfg
