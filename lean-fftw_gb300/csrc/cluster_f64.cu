// One small binary64 transform spread over a thread-block cluster (the latency path).
//
// On GB300 a binary64 warp instruction holds its SM sub-partition's FP64 pipe for 64 cycles
// however few lanes are active, so a butterfly evaluated by one thread costs its operation
// count times 64 cycles: a lone 1024-point transform on one CTA takes 21-27 us whatever its
// radices.  Here every butterfly is evaluated by a group of W lanes, level by level of its
// operation DAG, one operation per lane per level (lfg/codegen/wide.py builds the schedules;
// a twiddled radix-16 butterfly is 208 operations but 8 levels), and the butterflies of a pass
// are spread over a cluster of up to 16 CTAs of 128 threads (one warp per SM sub-partition, so
// no two warps of a level share an FP64 pipe).  Each lane group keeps a value table in
// shared memory (1.0, -0.0, the kernel's constants, its inputs, one slot per operation); a
// level is, per lane, three table reads, one fused multiply-add and one table write, then a
// warp barrier.  Every operation is the fused multiply-add the straight-line codelet issues
// for it, on the same operands (a negation is a sign flip of the operand's bits), so the bits
// are the same as for every other kernel of the library with the same radix sequence.
//
// Everything a CTA reads besides the data -- each pass's geometry, its schedule and its
// twiddle table -- is one device image built when the plan is made; the kernel copies it into
// shared memory with one burst of asynchronous copies (the first pass's inputs are loaded from
// global memory meanwhile), so no pass waits on a dependent chain of parameter or table loads.
//
// Data movement between passes:
// * the first pass reads its butterflies' inputs from global memory, the last pass writes its
//   outputs straight to global memory;
// * every other pass reads its inputs from this CTA's shared memory and writes each output
//   into the shared memory of the one CTA whose lane group reads it in the next pass, then
//   the cluster barrier orders the passes.
//
// The cluster barrier is a hardware barrier of co-scheduled CTAs (no polling): every thread of
// every CTA reaches every barrier, and no CTA touches another's shared memory after the last
// one, so none exits while its memory is still being written.  In place is safe: every input
// is read in the first pass, before the barrier that precedes the first output store.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstring>

#include "generated/wide_f64.h"
#include "kernels.h"
#include "stockham_dev.cuh"

namespace cg = cooperative_groups;

namespace lfg {
using namespace dev;

namespace {

constexpr int kClusterThreads = 128;   // four warps: one per SM sub-partition
constexpr int kMaxCluster = 16;       // CTAs (a non-portable cluster size above 8)
constexpr int kClusterWarps = kClusterThreads / 32;
constexpr int kMaxInPerLane = 4;      // first-pass inputs one lane prefetches (2R / W <= 2)

// One pass as the kernel reads it (the head of the image).  Byte offsets are from the start
// of the image; tw = -1: an untwiddled pass.
struct PassLite {
  int R, MR, ns, nsg;
  unsigned fdns_m, fdns_l, fdmrn_m, fdmrn_l;   // divisors ns and the next pass's MR
  int mrn, lgpcn, tw, W;                       // next pass: MR, log2 groups per CTA per round
  int depth, n_in, n_consts, n_slots;
  int sdesc, sconst, sout, lw;                 // lw = log2 W
};
static_assert(sizeof(PassLite) % 16 == 0, "16-byte image blocks");

__device__ __forceinline__ void cp_async16_cl(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 16;" ::"r"(
                   (unsigned)__cvta_generic_to_shared(dst)), "l"(src) : "memory");
}

// value with its sign bit flipped when `neg` (the operand's exact negation)
__device__ __forceinline__ double flip(unsigned long long bits, unsigned long long neg) {
  return __longlong_as_double((long long)(bits ^ (neg << 63)));
}

__device__ __forceinline__ int fdiv2(int n, unsigned m, unsigned l) {
  return (int)((__umulhi(m, (unsigned)n) + (unsigned)n) >> l);
}

// Shared memory of each CTA: two buffers of the padded array, the image, the warps' value
// tables.  The direction is in the schedules and the twiddle tables.
template <int S>
__global__ void __launch_bounds__(kClusterThreads)
cluster_kernel_f64(const ClusterArgs a, const double2* in, double2* out) {
  extern __shared__ double2 smem_cl[];
  cg::cluster_group cluster = cg::this_cluster();
  const int N = a.N;
  const int PN = sub_pitch(N);
  const unsigned rank = cluster.block_rank();
  unsigned char* const IMG = reinterpret_cast<unsigned char*>(smem_cl + 2 * PN);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double* const Vw = reinterpret_cast<double*>(IMG + a.img_bytes) + warp * a.vwarp;
  const unsigned char* const img = static_cast<const unsigned char*>(a.img);
  for (int i = threadIdx.x; i < a.img_bytes / 16; i += kClusterThreads)
    cp_async16_cl(IMG + 16 * i, img + 16 * i);
  asm volatile("cp.async.commit_group;" ::: "memory");
  // the first pass's first round: its inputs, while the image arrives
  double vin[kMaxInPerLane];
  {
    const int W = a.W0, gpw = 32 / W, gi = lane / W, s = lane - gi * W, MR = N / a.R0;
    const int q = (int)rank * kClusterWarps * gpw + warp * gpw + gi;
    const double* gin = reinterpret_cast<const double*>(in);
#pragma unroll
    for (int u = 0; u < kMaxInPerLane; ++u) {
      const int i = s + u * W;
      vin[u] = (q < MR && i < a.nin0) ? gin[2 * (q + (i >> 1) * MR) + (i & 1)] : 0.0;
    }
  }
  asm volatile("cp.async.wait_group 0;" ::: "memory");
  __syncthreads();   // the image is visible to every thread
  const PassLite* const PL = reinterpret_cast<const PassLite*>(IMG);
  const bool unit = a.unit != 0;
  const double sc = a.scale;
  const int last = a.npass - 1;
  for (int t = 0; t <= last; ++t) {
    const PassLite& P = PL[t];
    const int R = P.R, MR = P.MR, ns = P.ns, nsg = P.nsg;
    const int W = P.W, gpw = 32 >> P.lw, gi = lane >> P.lw, s = lane & (W - 1);
    const int gpc = kClusterWarps * gpw;               // groups per CTA per round
    const int depth = P.depth, n_in = P.n_in, n_consts = P.n_consts;
    double* const V = Vw + gi * P.n_slots;
    unsigned long long* const Vb = reinterpret_cast<unsigned long long*>(V);
    const unsigned long long* const desc = reinterpret_cast<const unsigned long long*>(IMG + P.sdesc);
    const unsigned long long* const cst = reinterpret_cast<const unsigned long long*>(IMG + P.sconst);
    const unsigned* const outs = reinterpret_cast<const unsigned*>(IMG + P.sout);
    const double* const twp = reinterpret_cast<const double*>(IMG + (P.tw >= 0 ? P.tw : 0));
    // pass t writes buffer t mod 2 (of the consuming CTA) and reads the other one
    double2* const wbuf = smem_cl + ((t & 1) ? PN : 0);
    const double* const rbuf = reinterpret_cast<const double*>(smem_cl + ((t & 1) ? 0 : PN));
    const double* const gin = reinterpret_cast<const double*>(in);
    unsigned long long dl[kWideMaxDepth];
#pragma unroll
    for (int L = 0; L < kWideMaxDepth; ++L) dl[L] = L < depth ? desc[L * W + s] : 0ull;
    // the previous pass's outputs: the setup above reads only this CTA's image, so it
    // overlaps the cluster barrier
    if (t > 0) cluster.barrier_wait();
    bool first = true;
    for (int base = (int)rank * gpc; base + warp * gpw < MR; base += S * gpc, first = false) {
      const int q = base + warp * gpw + gi;            // this group's butterfly
      const bool valid = q < MR;
      const int b = fdiv2(q, P.fdns_m, P.fdns_l), k = q - b * ns;
      for (int i = s; i < n_consts; i += W) Vb[i] = cst[i];
      if (valid) {
        if (t == 0 && first) {
#pragma unroll
          for (int u = 0; u < kMaxInPerLane; ++u)
            if (s + u * W < n_in) V[n_consts + s + u * W] = vin[u];
        } else {
          for (int i = s; i < n_in; i += W) {
            double v;
            if (i < 2 * R) {
              const int e = q + (i >> 1) * MR;
              v = t == 0 ? gin[2 * e + (i & 1)] : rbuf[2 * spad(e) + (i & 1)];
            } else {
              const int r = (i - 2 * R) >> 1;
              v = twp[2 * (k + r * nsg) + (i & 1)];
            }
            V[n_consts + i] = v;
          }
        }
      }
      __syncwarp();
      // every lane issues every level (idle lanes write a scratch slot; a group past the
      // last butterfly computes values that are never stored)
#pragma unroll
      for (int L = 0; L < kWideMaxDepth; ++L) {
        if (L < depth) {
          const unsigned long long d = dl[L];
          const double x = flip(Vb[d & 1023ull], (d >> 30) & 1ull);
          const double y = V[(d >> 10) & 1023ull];
          const double z = flip(Vb[(d >> 20) & 1023ull], (d >> 31) & 1ull);
          V[(d >> 32) & 1023ull] = __fma_rn(x, y, z);
          __syncwarp();
        }
      }
      if (valid) {
        const int d0 = b * ns * R + k;
        for (int j = s; j < R; j += W) {
          const unsigned ore = outs[2 * j], oim = outs[2 * j + 1];
          const double2 v = make_double2(flip(Vb[ore & 0x7fffu], ore >> 15),
                                         flip(Vb[oim & 0x7fffu], oim >> 15));
          const int o = d0 + j * ns;
          if (t == last && last > 0) {
            out[o] = unit ? v : make_double2(__dmul_rn(v.x, sc), __dmul_rn(v.y, sc));
          } else if (S == 1) {
            wbuf[spad(o)] = v;
          } else {
            // the next pass's butterfly reading o, and the CTA that runs it
            const int qn = o - fdiv2(o, P.fdmrn_m, P.fdmrn_l) * P.mrn;
            const unsigned owner = (unsigned)(qn >> P.lgpcn) & (unsigned)(S - 1);
            *cluster.map_shared_rank(wbuf + spad(o), owner) = v;
          }
        }
      }
      __syncwarp();   // the value table is reused by the next round
    }
    // this pass's outputs are in place before the next pass reads them: arrive here, wait
    // after the next pass's setup
    if (t < last) cluster.barrier_arrive();
    else if (last == 0) cluster.sync();
  }
  if (last == 0) {   // S == 1: the buffer holds the whole result
    const double2* res = smem_cl;
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
      const double2 v = res[spad(i)];
      out[i] = unit ? v : make_double2(__dmul_rn(v.x, sc), __dmul_rn(v.y, sc));
    }
  }
}

template <int S>
cudaError_t launch_s(const ClusterArgs& a, const void* in, void* out, size_t smem,
                     cudaStream_t stream) {
  auto kern = cluster_kernel_f64<S>;
  // the shared-memory opt-in once per device (devices 0..63)
  static std::atomic<unsigned long long> opted{0};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const unsigned long long bit = dev < 64 ? 1ull << dev : 0;
  if (!bit || !(opted.load(std::memory_order_relaxed) & bit)) {
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemBudget);
    if (e != cudaSuccess) return e;
    if (S > 8) {
      e = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
      if (e != cudaSuccess) return e;
    }
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
  return cudaLaunchKernelEx(&cfg, kern, a, static_cast<const double2*>(in),
                            static_cast<double2*>(out));
}

const WideInfo& wide_info(bool fwd, int R, bool tw) { return kWideInfo[fwd ? 1 : 0][R][tw ? 1 : 0]; }

size_t align16(size_t n) { return (n + 15) & ~(size_t)15; }

}  // namespace

int cluster_size_f64(const GroupDesc& g) {
  if (g.M < 2 || g.M > kClusterMaxN || g.npass < 1 || g.npass > kMaxPass) return 0;
  int lanes = 0;
  for (int t = 0; t < g.npass; ++t) {
    const int R = g.pass[t].R;
    if (R < 2 || R > 16 || g.M % R) return 0;
    const WideInfo& w = wide_info(true, R, t > 0);
    if (w.W == 0) return 0;
    if (t == 0 && w.n_in > kMaxInPerLane * w.W) return 0;   // the first round's prefetch
    lanes = std::max(lanes, (g.M / R) * w.W);
  }
  int S = 1;
  while (S < kMaxCluster && S * kClusterThreads < lanes) S *= 2;
  // a one-pass transform stores from its own buffer: one CTA
  return g.npass == 1 && S > 1 ? 0 : S;
}

size_t build_cluster_image_f64(const GroupDesc& g, bool fwd, const double* tw_values,
                               const size_t* tw_offset, std::vector<unsigned char>& img,
                               ClusterArgs* args) {
  const int S = cluster_size_f64(g);
  if (S == 0) return 0;
  const int np = g.npass;
  // layout: pass heads, each pass's schedule (descriptors, constants, output slots), then
  // each twiddled pass's table (interleaved pairs)
  size_t off = align16(np * sizeof(PassLite));
  std::vector<PassLite> pl(np);
  std::vector<size_t> sd(np), sc(np), so(np), st(np, 0);
  int vwarp = 0;
  for (int t = 0; t < np; ++t) {
    const WideInfo& w = wide_info(fwd, g.pass[t].R, t > 0);
    sd[t] = off;
    off = align16(off + (size_t)w.depth * w.W * 8);
    sc[t] = off;
    off = align16(off + (size_t)w.n_consts * 8);
    so[t] = off;
    off = align16(off + (size_t)2 * g.pass[t].R * 4);
    vwarp = std::max(vwarp, (32 / w.W) * w.n_slots);
  }
  for (int t = 1; t < np; ++t) {
    st[t] = off;
    off = align16(off + (size_t)2 * (g.pass[t].R - 1) * g.pass[t].ns_g * 8);
  }
  img.assign(off, 0);
  for (int t = 0; t < np; ++t) {
    const PassDesc& pd = g.pass[t];
    const WideInfo& w = wide_info(fwd, pd.R, t > 0);
    PassLite& P = pl[t];
    P.R = pd.R;
    P.MR = g.M / pd.R;
    P.ns = pd.ns_loc;
    P.nsg = pd.ns_g;
    const FastDiv fns = make_fastdiv(pd.ns_loc);
    P.fdns_m = fns.m;
    P.fdns_l = fns.l;
    const int tn = t + 1 < np ? t + 1 : t;
    const WideInfo& wn = wide_info(fwd, g.pass[tn].R, tn > 0);
    P.mrn = g.M / g.pass[tn].R;
    const FastDiv fmr = make_fastdiv(P.mrn);
    P.fdmrn_m = fmr.m;
    P.fdmrn_l = fmr.l;
    int lwn = 0;
    while ((1 << lwn) < wn.W) ++lwn;
    P.lgpcn = 2 + 5 - lwn;   // log2(kClusterWarps * 32 / W_next)
    static_assert(kClusterWarps == 4, "lgpcn assumes four warps per CTA");
    P.tw = t > 0 ? (int)st[t] : -1;
    P.W = w.W;
    P.depth = w.depth;
    P.n_in = w.n_in;
    P.n_consts = w.n_consts;
    P.n_slots = w.n_slots;
    P.sdesc = (int)sd[t];
    P.sconst = (int)sc[t];
    P.sout = (int)so[t];
    P.lw = 0;
    while ((1 << P.lw) < w.W) ++P.lw;
    std::memcpy(img.data() + sd[t], kWideDesc + w.desc_off, (size_t)w.depth * w.W * 8);
    std::memcpy(img.data() + sc[t], kWideConst + w.const_off, (size_t)w.n_consts * 8);
    std::memcpy(img.data() + so[t], kWideOut + w.out_off, (size_t)2 * pd.R * 4);
    if (t > 0)
      std::memcpy(img.data() + st[t], tw_values + tw_offset[t],
                  (size_t)2 * (pd.R - 1) * pd.ns_g * 8);
  }
  std::memcpy(img.data(), pl.data(), np * sizeof(PassLite));
  const WideInfo& w0 = wide_info(fwd, g.pass[0].R, false);
  *args = ClusterArgs{};
  args->img_bytes = (int)off;
  args->N = g.M;
  args->npass = np;
  args->vwarp = vwarp;
  args->R0 = g.pass[0].R;
  args->W0 = w0.W;
  args->nin0 = w0.n_in;
  args->S = S;
  return off;
}

size_t cluster_smem_bytes_f64(const ClusterArgs& a) {
  return 2 * (size_t)sub_pitch(a.N) * sizeof(double2) + (size_t)a.img_bytes +
         (size_t)kClusterWarps * a.vwarp * sizeof(double);
}

cudaError_t launch_cluster_f64(const ClusterArgs& args, double scale, const void* in, void* out,
                               cudaStream_t stream) {
  ClusterArgs a = args;
  a.scale = scale;
  a.unit = scale == 1.0 ? 1 : 0;
  const size_t smem = cluster_smem_bytes_f64(a);
  if (smem > kSmemBudget || !a.img) return cudaErrorInvalidValue;
  switch (a.S) {
    case 1: return launch_s<1>(a, in, out, smem, stream);
    case 2: return launch_s<2>(a, in, out, smem, stream);
    case 4: return launch_s<4>(a, in, out, smem, stream);
    case 8: return launch_s<8>(a, in, out, smem, stream);
    case 16: return launch_s<16>(a, in, out, smem, stream);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace lfg
