// Batched one-butterfly transforms: N = R <= 16 points, a single untwiddled pass.
//
// A plan of such a size is one codelet per transform, so its kernel is a copy with a little
// arithmetic: memory-bound in binary32, and in binary64 bound by memory for N <= 4 and by the
// FP64 pipe above.  The shared-memory group kernel moves each byte through a CTA-wide tile
// and two barriers per tile, which leaves these sizes at 35-60 % of HBM.  Here each warp works
// on its own chunk of transforms with warp-level synchronisation only:
//
//   1. the chunk (32 K transforms, K = 256 / (R x element bytes), so that every lane has about
//      256 bytes in flight) is read with coalesced loads -- consecutive lanes take consecutive elements
//      of a transform when elements are contiguous, else the same element of consecutive
//      transforms -- into the warp's tile (layout: small_slot below, conflict-free for the
//      staging and for the lane-strided reads and writes of step 2);
//   2. each lane runs the codelet on K transforms of the tile, in place (scaled on the way
//      out when the plan's scale is not 1, as the group kernel's stores do);
//   3. the chunk is written back with the loads' ordering.
//
// The butterflies are the generated codelets of the group kernels, so the results are the
// same bits.  In place is safe: a warp reads its whole chunk before it writes any of it, and
// chunks are disjoint.
#include <cuda_runtime.h>

#include <algorithm>

#include "kernels.h"
#include "stockham_dev.cuh"

namespace lfg {
using namespace dev;
namespace {

constexpr int kSmallThreads = 256;
constexpr int kSmallWarps = kSmallThreads / 32;

// transforms per lane: about 256 bytes of loads in flight per lane (16 binary64 or 32
// binary32 complex elements)
__host__ __device__ constexpr int small_k(int R, int elem_bytes) {
  return R * elem_bytes >= 256 ? 1 : 256 / (R * elem_bytes);
}
// Tile layout: transform t's element r at t * pitch + slot(t, r).  Binary64 with power-of-two
// R: no padding, the element index XOR-swizzled by a function of t so that both the staging
// accesses (consecutive elements) and the per-lane reads (one transform per lane, stride R)
// hit distinct banks (N = 2: 0.430 -> 0.367 ms with the 3-CTA register cap below).  Otherwise
// an odd pitch R | 1 and no swizzle (binary32 measured slower swizzled: N = 8 0.403 -> 0.449
// ms, the extra index arithmetic spilling at the 128-register cap).
__host__ __device__ constexpr bool small_swizzled(int R, int elem_bytes) {
  return elem_bytes == 16 && (R & (R - 1)) == 0;
}
__host__ __device__ constexpr int small_pitch(int R, int elem_bytes) {
  return small_swizzled(R, elem_bytes) ? R : (R | 1);
}
// U = 128-byte bank row / element size: the accesses of one shared-memory wavefront
template <int R, int U>
__device__ __forceinline__ int small_slot(int t, int r) {
  if constexpr (small_swizzled(R, 128 / U)) return r ^ ((t / (U > R ? U / R : 1)) & (R - 1));
  else return r;
}

// binary64 R <= 8: three CTAs per SM (80 registers, no spills; more loads in flight); binary64
// R = 16: one (224 registers; at 128 it spills, and 4 % slower than the group kernel, 1.163
// against 1.213 ms for 2^22 lines); else two
template <class T, bool FWD, int R>
__global__ void __launch_bounds__(kSmallThreads,
                                  (sizeof(T) == 8 && R <= 8) ? 3 : (sizeof(T) == 8 && R == 16) ? 1 : 2)
small_kernel(const GroupDesc g, const typename Prec<T>::C* in, typename Prec<T>::C* out) {
  using P = Prec<T>;
  using Cx = typename P::C;
  constexpr int K = small_k(R, (int)sizeof(Cx)), TPW = 32 * K, PT = small_pitch(R, (int)sizeof(Cx));
  constexpr int U = 128 / (int)sizeof(Cx);
  extern __shared__ double2 small_smem[];
  const int lane = threadIdx.x & 31;
  Cx* const tile = reinterpret_cast<Cx*>(small_smem) + (threadIdx.x >> 5) * (TPW * PT);
  const int64_t ntr = g.total_sub;
  const int64_t nchunks = (ntr + TPW - 1) / TPW;
  const int64_t wstride = (int64_t)gridDim.x * kSmallWarps;
  const int64_t il = g.in_line, ie = g.in_elem, ol = g.out_line, oe = g.out_elem;
  const bool in_rfast = ie == 1, out_rfast = oe == 1;
  const bool in_packed = in_rfast && il == R, out_packed = out_rfast && ol == R;   // back to back
  const bool unit = g.unit_scale != 0;
  const T sc = sizeof(T) == 4 ? (T)g.scale_f32 : (T)g.scale;
  T one, nz;
  P::units(one, nz);
  for (int64_t ch = (int64_t)blockIdx.x * kSmallWarps + (threadIdx.x >> 5); ch < nchunks; ch += wstride) {
    const int64_t t0 = ch * TPW;
    const int nt = (int)min((int64_t)TPW, ntr - t0);
    const Cx* src = in + t0 * il;
    Cx* dst = out + t0 * ol;
    if (in_packed) {
#pragma unroll
      for (int k = 0; k < R * K; ++k) {
        const int e = k * 32 + lane;
        if (e < nt * R) tile[(e / R) * PT + small_slot<R, U>(e / R, e % R)] = src[e];
      }
    } else {
#pragma unroll
      for (int k = 0; k < R * K; ++k) {
        const int e = k * 32 + lane;
        const int t = in_rfast ? e / R : e % TPW;
        const int r = in_rfast ? e - t * R : e / TPW;
        if (t < nt) tile[t * PT + small_slot<R, U>(t, r)] = src[(int64_t)t * il + (int64_t)r * ie];
      }
    }
    __syncwarp();
#pragma unroll 1
    for (int k = 0; k < K; ++k) {
      const int t = k * 32 + lane;
      Cx* const v = tile + t * PT;
      T x[2 * R], y[2 * R];
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const Cx a = v[small_slot<R, U>(t, r)];
        x[2 * r] = a.x;
        x[2 * r + 1] = a.y;
      }
      P::template Bfly<FWD, R, false>::run(x, y, one, nz);
#pragma unroll
      for (int r = 0; r < R; ++r)
        v[small_slot<R, U>(t, r)] = unit ? P::mk(y[2 * r], y[2 * r + 1])
                                         : P::mk(P::mul(y[2 * r], sc), P::mul(y[2 * r + 1], sc));
    }
    __syncwarp();
    if (out_packed) {
#pragma unroll
      for (int k = 0; k < R * K; ++k) {
        const int e = k * 32 + lane;
        if (e < nt * R) dst[e] = tile[(e / R) * PT + small_slot<R, U>(e / R, e % R)];
      }
    } else {
#pragma unroll
      for (int k = 0; k < R * K; ++k) {
        const int e = k * 32 + lane;
        const int t = out_rfast ? e / R : e % TPW;
        const int r = out_rfast ? e - t * R : e / TPW;
        if (t < nt) dst[(int64_t)t * ol + (int64_t)r * oe] = tile[t * PT + small_slot<R, U>(t, r)];
      }
    }
    __syncwarp();   // the tile is refilled by the warp's next chunk
  }
}

template <class T>
size_t small_smem(int R) {
  constexpr int es = (int)sizeof(typename Prec<T>::C);
  return (size_t)kSmallWarps * 32 * small_k(R, es) * small_pitch(R, es) * es;
}

template <class T, bool FWD>
const void* small_fn(int R) {
  switch (R) {
#define LFG_SMALL_CASE(RR) \
  case RR: return (const void*)small_kernel<T, FWD, RR>;
    LFG_SMALL_CASE(2)
    LFG_SMALL_CASE(3)
    LFG_SMALL_CASE(4)
    LFG_SMALL_CASE(5)
    LFG_SMALL_CASE(6)
    LFG_SMALL_CASE(7)
    LFG_SMALL_CASE(8)
    LFG_SMALL_CASE(9)
    LFG_SMALL_CASE(10)
    LFG_SMALL_CASE(11)
    LFG_SMALL_CASE(12)
    LFG_SMALL_CASE(13)
    LFG_SMALL_CASE(14)
    LFG_SMALL_CASE(15)
    LFG_SMALL_CASE(16)
#undef LFG_SMALL_CASE
    default: return nullptr;
  }
}

const void* small_kernel_fn(int precision, bool fwd, int R) {
  if (precision == 0) return fwd ? small_fn<double, true>(R) : small_fn<double, false>(R);
  return fwd ? small_fn<float, true>(R) : small_fn<float, false>(R);
}

size_t small_smem_bytes(int precision, int R) {
  return precision == 0 ? small_smem<double>(R) : small_smem<float>(R);
}

}  // namespace

bool small_kernel_applies(const GroupDesc& g) {
  return g.npass == 1 && g.nsub == 1 && g.M >= 2 && g.M <= kSmallMaxN && g.pass[0].R == g.M &&
         g.pass[0].tw == nullptr && g.total_sub > 0;
}

cudaError_t prepare_small_kernels() {
  for (int prec = 0; prec < 2; ++prec)
    for (int fwd = 0; fwd < 2; ++fwd)
      for (int R = 2; R <= kSmallMaxN; ++R) {
        const size_t s = small_smem_bytes(prec, R);
        if (s <= 48 * 1024) continue;
        cudaError_t e = cudaFuncSetAttribute(small_kernel_fn(prec, fwd != 0, R),
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s);
        if (e != cudaSuccess) return e;
      }
  return cudaSuccess;
}

unsigned small_grid(const GroupDesc& g, int precision) {
  const int R = g.M;
  const void* fn = small_kernel_fn(precision, true, R);
  int dev = 0, sms = 1, per_sm = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kSmallThreads,
                                                    small_smem_bytes(precision, R)) != cudaSuccess ||
      per_sm < 1)
    per_sm = 1;
  const int64_t tpb = (int64_t)kSmallWarps * 32 * small_k(R, precision == 0 ? 16 : 8);
  const int64_t need = (g.total_sub + tpb - 1) / tpb;
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(need, (int64_t)sms * per_sm));
}

cudaError_t launch_small(const GroupDesc& gd, int precision, bool fwd, const void* in, void* out,
                         unsigned grid, cudaStream_t stream) {
  if (!small_kernel_applies(gd)) return cudaErrorInvalidValue;
  GroupDesc g = gd;
  set_divisors(g);
  const int R = g.M;
  const size_t smem = small_smem_bytes(precision, R);
  void* args[] = {(void*)&g, (void*)&in, (void*)&out};
  return cudaLaunchKernel(small_kernel_fn(precision, fwd, R), dim3(grid), dim3(kSmallThreads), args,
                          smem, stream);
}

}  // namespace lfg
