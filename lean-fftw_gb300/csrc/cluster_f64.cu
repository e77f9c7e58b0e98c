// One small binary64 transform spread over a thread-block cluster (the latency path).
//
// A lone transform of N <= kClusterMaxN points gives one CTA of the group kernel only a few
// warps per pass, and on GB300 each warp's binary64 instruction holds its SM sub-partition's
// FP64 pipe for 64 cycles: a radix-16 pass of a 1024-point transform is 208 such instructions
// in a row on one warp, about 6 us, whatever the other sub-partitions do.  Here a cluster of
// S CTAs (S SMs, four warps each, one per sub-partition) shares the transform so that every
// warp of a pass owns at most one butterfly per thread, and every CTA keeps a full copy of the
// array in its own shared memory: a pass reads its butterflies' inputs locally and writes each
// output into the next buffer of every CTA of the cluster (distributed shared memory), then
// the cluster barrier orders the pass.  The passes perform the reference codelets exactly as
// the group kernel does (same DAGs, same twiddle tables, same operand order), so the bits are
// the same as for any other kernel of the library with the same radix sequence.
//
// The cluster barrier is a hardware barrier of co-scheduled CTAs (no polling): every thread of
// every CTA reaches every barrier, and no CTA touches another's shared memory after the last
// one, so none exits while its memory is still being written.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>

#include "stockham_dev.cuh"

namespace cg = cooperative_groups;

namespace lfg {
using namespace dev;
namespace {

constexpr int kClusterThreads = 128;   // one warp per SM sub-partition

// One pass over the whole transform: butterflies q = q0, q0 + qstep, ... of N / R, inputs from
// the local buffer `src` (padded layout spad), twiddles from the local table copy, outputs to
// the same position of the next buffer in every CTA of the cluster.
template <bool FWD, int R, bool TW, int S>
__device__ __forceinline__ void cluster_pass(const double2* __restrict__ src, double2* const* dst,
                                             int N, const PassDesc& pd,
                                             const double2* __restrict__ tw, int q0, int qstep) {
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
      const double2 v = src[spad(q + r * MR)];
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
      const int o = spad(d0 + r * ns);
#pragma unroll
      for (int s = 0; s < S; ++s) dst[s][o] = v;
    }
  }
}

template <bool FWD, int S>
__device__ __forceinline__ void cluster_pass_any(const double2* src, double2* const* dst, int N,
                                                 const PassDesc& pd, const double2* tw, int q0,
                                                 int qstep) {
#define LFG_CPASS(RR)                                                              \
  case RR:                                                                         \
    if (tw) cluster_pass<FWD, RR, true, S>(src, dst, N, pd, tw, q0, qstep);        \
    else cluster_pass<FWD, RR, false, S>(src, dst, N, pd, tw, q0, qstep);          \
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
  double2* A = smem_cl;
  double2* B = smem_cl + PN;
  double2* T = smem_cl + 2 * PN;
  // the input line and the twiddle tables, into this CTA's shared memory (in == out is
  // allowed: every CTA has read the input before the first barrier, and the output is
  // written after the last)
  for (int i = threadIdx.x; i < N; i += blockDim.x) A[spad(i)] = in[i];
  for (int i = threadIdx.x; i < tw_len; i += blockDim.x) T[i] = tw_base[i];
  // the same buffers in every CTA of the cluster
  double2* dA[S];
  double2* dB[S];
#pragma unroll
  for (int s = 0; s < S; ++s) {
    dA[s] = cluster.map_shared_rank(A, s);
    dB[s] = cluster.map_shared_rank(B, s);
  }
  cluster.sync();   // every copy loaded before any remote write
  const int q0 = rank * kClusterThreads + threadIdx.x;
  const int qstep = S * kClusterThreads;
  bool in_a = true;
  for (int t = 0; t < g.npass; ++t) {
    const PassDesc& pd = g.pass[t];
    const double2* tw = pd.tw ? T + (static_cast<const double2*>(pd.tw) - tw_base) : nullptr;
    cluster_pass_any<FWD, S>(in_a ? A : B, in_a ? dB : dA, N, pd, tw, q0, qstep);
    cluster.sync();   // the pass's outputs are in every CTA before the next pass reads them
    in_a = !in_a;
  }
  // every CTA holds the whole result: each stores its share
  const double2* res = in_a ? A : B;
  const int per = (N + S - 1) / S;
  const int lo = rank * per, hi = min(N, lo + per);
  const double sc = g.scale;
  for (int i = lo + (int)threadIdx.x; i < hi; i += blockDim.x) {
    const double2 v = res[spad(i)];
    out[i] = g.unit_scale ? v : make_double2(__dmul_rn(v.x, sc), __dmul_rn(v.y, sc));
  }
}

template <bool FWD, int S>
cudaError_t launch_s(const GroupDesc& g, const void* in, void* out, const double2* tw_base,
                     int tw_len, size_t smem, cudaStream_t stream) {
  auto kern = cluster_kernel_f64<FWD, S>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
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
  return S;
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
