// One small binary64 transform spread over a thread-block cluster (the latency path).
//
// A lone transform of N <= kClusterMaxN points gives one CTA of the group kernel only a few
// warps per pass, and on GB300 each warp's binary64 instruction holds its SM sub-partition's
// FP64 pipe for 64 cycles: a radix-16 pass of a 1024-point transform is 208 such instructions
// in a row on one warp, about 6 us, whatever the other sub-partitions do.  Here a cluster of
// S CTAs (S SMs, four warps each, one per sub-partition) shares the transform so that every
// warp of a pass owns at most one butterfly per thread, and the planner picks radices for the
// serial operation count of one butterfly per pass (radix 4 where the size allows).
//
// Data movement is kept off the critical path:
// * the first pass reads its butterflies' inputs straight from global memory, and the last
//   pass writes its outputs straight to global memory (no copy loops before or after);
// * every other pass reads its inputs from this CTA's shared memory and writes each output
//   into the shared memory of the one CTA whose thread reads it in the next pass (butterfly
//   q of a pass runs on CTA (q / 128) mod S), then the cluster barrier orders the passes;
// * the twiddle tables are copied into each CTA's shared memory asynchronously while the
//   first (untwiddled) pass computes.
// The passes perform the reference codelets exactly as the group kernel does (same DAGs,
// same twiddle tables, same operand order), so the bits are the same as for any other kernel
// of the library with the same radix sequence.
//
// The cluster barrier is a hardware barrier of co-scheduled CTAs (no polling): every thread of
// every CTA reaches every barrier, and no CTA touches another's shared memory after the last
// one, so none exits while its memory is still being written.  In place is safe: every input
// is read in the first pass, before the barrier that precedes the first output store.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>

#include "stockham_dev.cuh"

namespace cg = cooperative_groups;

namespace lfg {
using namespace dev;
namespace {

constexpr int kClusterThreads = 128;   // one warp per SM sub-partition

__device__ __forceinline__ void cp_async16_cl(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 16;" ::"r"(
                   (unsigned)__cvta_generic_to_shared(dst)), "l"(src) : "memory");
}

// Pass kinds: the first pass (untwiddled; inputs from global memory, outputs to the consuming
// CTA's buffer), a middle pass (twiddled; local buffer to the consuming CTA's buffer) and the
// last pass (twiddled; local buffer to global memory, scaled).
enum PassKind { kFirst = 0, kMiddle = 1, kLast = 2 };

// One pass over the whole transform: butterflies q = q0, q0 + qstep, ... of N / R.  `mrn` and
// `fdn`: butterflies per line of the next pass and its divisor (output o is read there by
// butterfly o mod mrn).
template <bool FWD, int R, int KIND, int S>
__device__ __forceinline__ void cluster_pass(const double2* __restrict__ gin, const double2* src,
                                             double2* dst, double2* __restrict__ gout, int N,
                                             const PassDesc& pd, int mrn, FastDiv fdn,
                                             const double2* tw, int q0, int qstep, bool unit,
                                             double sc) {
  constexpr bool TW = KIND != kFirst;
  const int MR = N / R;
  const int ns = pd.ns_loc;
  const int nsg = pd.ns_g;
  const FastDiv fd_ns = pd.fd_ns;
  double one, nz;
  Prec<double>::units(one, nz);
  for (int q = q0; q < MR; q += qstep) {
    double x[TW ? 4 * R - 2 : 2 * R];
    double y[2 * R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const double2 v = KIND == kFirst ? gin[q + r * MR] : src[spad(q + r * MR)];
      x[2 * r] = v.x;
      x[2 * r + 1] = v.y;
    }
    const int b = fdiv(q, fd_ns);
    const int k = q - b * ns;
    if (TW) {
#pragma unroll
      for (int r = 0; r < R - 1; ++r) {
        const double2 v = tw[k + r * nsg];
        x[2 * R + 2 * r] = v.x;
        x[2 * R + 2 * r + 1] = v.y;
      }
    }
    BflyD<FWD, R, TW>::run(x, y, one, nz);
    const int d0 = b * ns * R + k;
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const double2 v = make_double2(y[2 * r], y[2 * r + 1]);
      const int o = d0 + r * ns;
      if (KIND == kLast) {
        gout[o] = unit ? v : make_double2(__dmul_rn(v.x, sc), __dmul_rn(v.y, sc));
      } else if (S == 1) {
        dst[spad(o)] = v;
      } else {
        const int qn = o - fdiv(o, fdn) * mrn;   // the next pass's butterfly reading o
        const unsigned owner = (unsigned)(qn >> 7) & (unsigned)(S - 1);
        *cg::this_cluster().map_shared_rank(dst + spad(o), owner) = v;
      }
    }
  }
}

template <bool FWD, int S>
__device__ __forceinline__ void cluster_pass_any(int kind, const double2* gin, const double2* src,
                                                 double2* dst, double2* gout, int N,
                                                 const PassDesc& pd, int mrn, FastDiv fdn,
                                                 const double2* tw, int q0, int qstep, bool unit,
                                                 double sc) {
#define LFG_CPASS(RR)                                                                          \
  case RR:                                                                                     \
    if (kind == kFirst)                                                                        \
      cluster_pass<FWD, RR, kFirst, S>(gin, src, dst, gout, N, pd, mrn, fdn, tw, q0, qstep,    \
                                       unit, sc);                                              \
    else if (kind == kMiddle)                                                                  \
      cluster_pass<FWD, RR, kMiddle, S>(gin, src, dst, gout, N, pd, mrn, fdn, tw, q0, qstep,   \
                                        unit, sc);                                             \
    else                                                                                       \
      cluster_pass<FWD, RR, kLast, S>(gin, src, dst, gout, N, pd, mrn, fdn, tw, q0, qstep,     \
                                      unit, sc);                                               \
    break;
  switch (pd.R) {
    LFG_CPASS(2)
    LFG_CPASS(3)
    LFG_CPASS(4)
    LFG_CPASS(5)
    LFG_CPASS(6)
    LFG_CPASS(7)
    LFG_CPASS(8)
    LFG_CPASS(9)
    LFG_CPASS(10)
    LFG_CPASS(11)
    LFG_CPASS(12)
    LFG_CPASS(13)
    LFG_CPASS(14)
    LFG_CPASS(15)
    LFG_CPASS(16)
    default: break;   // rejected by the planner
  }
#undef LFG_CPASS
}

// Shared memory of each CTA: two buffers of the padded array, then the pass twiddle tables
// (the plan's table range [tw_base, tw_base + tw_len) copied whole).
template <bool FWD, int S>
__global__ void __launch_bounds__(kClusterThreads)
cluster_kernel_f64(const GroupDesc g, const double2* in, double2* out,
                   const double2* __restrict__ tw_base, int tw_len) {
  extern __shared__ double2 smem_cl[];
  cg::cluster_group cluster = cg::this_cluster();
  const int N = g.M;
  const int PN = sub_pitch(N);
  const int rank = (int)cluster.block_rank();
  double2* T = smem_cl + 2 * PN;
  // the twiddle tables arrive while the first pass computes (it needs none)
  for (int i = threadIdx.x; i < tw_len; i += blockDim.x) cp_async16_cl(T + i, tw_base + i);
  asm volatile("cp.async.commit_group;" ::: "memory");
  const int q0 = rank * kClusterThreads + threadIdx.x;
  const int qstep = S * kClusterThreads;
  const bool unit = g.unit_scale != 0;
  const double sc = g.scale;
  const int last = g.npass - 1;
  for (int t = 0; t <= last; ++t) {
    const PassDesc& pd = g.pass[t];
    const double2* tw = pd.tw ? T + (static_cast<const double2*>(pd.tw) - tw_base) : nullptr;
    // a one-pass transform writes its buffer and stores it below (in place stays safe)
    const int kind = t == 0 ? kFirst : (t == last ? kLast : kMiddle);
    const PassDesc& pn = g.pass[t < last ? t + 1 : t];
    // pass t writes buffer t mod 2 and reads the other one
    double2* const wbuf = smem_cl + ((t & 1) ? PN : 0);
    const double2* const rbuf = smem_cl + ((t & 1) ? 0 : PN);
    cluster_pass_any<FWD, S>(kind, in, rbuf, wbuf, out, N, pd, N / pn.R, pn.fd_mr, tw, q0,
                             qstep, unit, sc);
    if (t < last || last == 0) {
      if (t == 0) asm volatile("cp.async.wait_group 0;" ::: "memory");
      cluster.sync();   // this pass's outputs are in place before the next pass reads them
    }
  }
  if (last == 0) {   // S == 1: the buffer holds the whole result
    const double2* res = smem_cl;
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
      const double2 v = res[spad(i)];
      out[i] = unit ? v : make_double2(__dmul_rn(v.x, sc), __dmul_rn(v.y, sc));
    }
  }
}

template <bool FWD, int S>
cudaError_t launch_s(const GroupDesc& g, const void* in, void* out, const double2* tw_base,
                     int tw_len, size_t smem, cudaStream_t stream) {
  auto kern = cluster_kernel_f64<FWD, S>;
  // the shared-memory opt-in once per device (devices 0..63)
  static std::atomic<unsigned long long> opted{0};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const unsigned long long bit = dev < 64 ? 1ull << dev : 0;
  if (!bit || !(opted.load(std::memory_order_relaxed) & bit)) {
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)(kSmemBudget));
    if (e != cudaSuccess) return e;
    opted.fetch_or(bit, std::memory_order_relaxed);
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(S, 1, 1);
  cfg.blockDim = dim3(kClusterThreads, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = S;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kern, g, static_cast<const double2*>(in),
                            static_cast<double2*>(out), tw_base, tw_len);
}

}  // namespace

int cluster_size_f64(const GroupDesc& g) {
  if (g.M < 2 || g.M > kClusterMaxN || g.npass < 1) return 0;
  int widest = 0;
  for (int t = 0; t < g.npass; ++t) widest = std::max(widest, g.M / g.pass[t].R);
  int S = 1;
  while (S < 8 && S * kClusterThreads < widest) S *= 2;
  // a one-pass transform stores from its own buffer: one CTA
  return g.npass == 1 && S > 1 ? 0 : S;
}

size_t cluster_smem_bytes_f64(const GroupDesc& g, int tw_len) {
  return (2 * (size_t)sub_pitch(g.M) + (size_t)tw_len) * sizeof(double2);
}

cudaError_t launch_cluster_f64(const GroupDesc& gd, bool fwd, const void* in, void* out,
                               const void* tw_base, int tw_len, cudaStream_t stream) {
  GroupDesc g = gd;
  set_divisors(g);
  const int S = cluster_size_f64(g);
  if (S == 0) return cudaErrorInvalidValue;
  const size_t smem = cluster_smem_bytes_f64(g, tw_len);
  if (smem > kSmemBudget) return cudaErrorInvalidValue;
  const double2* tw = static_cast<const double2*>(tw_base);
  switch (S) {
    case 1: return fwd ? launch_s<true, 1>(g, in, out, tw, tw_len, smem, stream)
                       : launch_s<false, 1>(g, in, out, tw, tw_len, smem, stream);
    case 2: return fwd ? launch_s<true, 2>(g, in, out, tw, tw_len, smem, stream)
                       : launch_s<false, 2>(g, in, out, tw, tw_len, smem, stream);
    case 4: return fwd ? launch_s<true, 4>(g, in, out, tw, tw_len, smem, stream)
                       : launch_s<false, 4>(g, in, out, tw, tw_len, smem, stream);
    default: return fwd ? launch_s<true, 8>(g, in, out, tw, tw_len, smem, stream)
                        : launch_s<false, 8>(g, in, out, tw, tw_len, smem, stream);
  }
}

}  // namespace lfg
