// Batched small transforms: one-butterfly sizes (N = R <= 16 points, a single untwiddled pass)
// in both precisions, and binary32 plans of two passes up to 32 points.
//
// A one-butterfly plan is one codelet per transform, so its kernel is a copy with a little
// arithmetic: memory-bound in binary32, and in binary64 bound by memory for N <= 4 and by the
// FP64 pipe above.  The shared-memory group kernel moves each byte through a CTA-wide tile
// and two barriers per tile, which leaves these sizes at 35-60 % of HBM.  Here each warp works
// on its own chunk of transforms with warp-level synchronisation only:
//
//   1. the chunk (32 K transforms, K = 256 / (N x element bytes), so that every lane has about
//      256 bytes in flight) is read with coalesced loads -- consecutive lanes take consecutive
//      elements of a transform when elements are contiguous, else the same element of
//      consecutive transforms -- into the warp's tile (layout: small_slot below,
//      conflict-free for the staging and for the lane-strided reads and writes of step 2);
//   2. each lane runs the plan on K transforms of the tile: the codelet in place (scaled on
//      the way out when the plan's scale is not 1, as the group kernel's stores do), or the
//      two passes between the warp's two tiles;
//   3. the chunk is written back with the loads' ordering.
//
// The butterflies are the generated codelets of the group kernels and the passes follow the
// same Stockham schedule, so the results are the same bits.  In place is safe: a warp reads
// its whole chunk before it writes any of it, and chunks are disjoint.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>

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

// Lane work of a one-pass plan: the codelet on transform t of the tile, in place (scaled on the
// way out when the plan's scale is not 1, as the group kernel's stores do).
template <class T, bool FWD, int R, int U, int PT>
__device__ __forceinline__ void small_onepass(typename Prec<T>::C* tile, int t, T one, T nz, bool unit,
                                              T sc) {
  using P = Prec<T>;
  using Cx = typename P::C;
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

// The warp's stores of a chunk of nt transforms (K per lane) from its tile to dst, in the
// loads' ordering: consecutive lanes on consecutive elements of a transform when the output's
// elements are contiguous, else on the same element of consecutive transforms.
template <int R, int U, int PT, int K, class Cx>
__device__ __forceinline__ void small_store(const Cx* tile, Cx* dst, int nt, int lane, bool packed,
                                            bool rfast, int64_t ol, int64_t oe) {
  constexpr int TPW = 32 * K;
  if (packed) {
#pragma unroll
    for (int k = 0; k < R * K; ++k) {
      const int e = k * 32 + lane;
      if (e < nt * R) dst[e] = tile[(e / R) * PT + small_slot<R, U>(e / R, e % R)];
    }
  } else {
#pragma unroll
    for (int k = 0; k < R * K; ++k) {
      const int e = k * 32 + lane;
      const int t = rfast ? e / R : e % TPW;
      const int r = rfast ? e - t * R : e / TPW;
      if (t < nt) dst[(int64_t)t * ol + (int64_t)r * oe] = tile[t * PT + small_slot<R, U>(t, r)];
    }
  }
}

// The kernel for a plan of radix R0 (R1 = 1), or of radices R0 then R1 (binary32, N = R0 R1
// <= 32 points: two passes, out of place between the warp's two tiles).  Binary64 R0 <= 8:
// three CTAs per SM (80 registers, no spills; more loads in flight); binary64 R0 = 16: one (224
// registers; at 128 it spills, and 4 % slower than the group kernel, 1.163 against 1.213 ms
// for 2^22 lines); else two.
template <class T, bool FWD, int R0, int R1>
__global__ void __launch_bounds__(kSmallThreads,
                                  (sizeof(T) == 8 && R0 <= 8) ? 3 : (sizeof(T) == 8 && R0 == 16) ? 1 : 2)
small_kernel(const GroupDesc g, const typename Prec<T>::C* in, typename Prec<T>::C* out) {
  using P = Prec<T>;
  using Cx = typename P::C;
  constexpr int R = R0 * R1;   // points per transform
  constexpr int K = small_k(R, (int)sizeof(Cx)), TPW = 32 * K, PT = small_pitch(R, (int)sizeof(Cx));
  constexpr int U = 128 / (int)sizeof(Cx);
  constexpr int NT = R1 > 1 ? 2 : 1;   // tiles per warp
  extern __shared__ double2 small_smem[];
  const int lane = threadIdx.x & 31;
  Cx* const tile = reinterpret_cast<Cx*>(small_smem) + (threadIdx.x >> 5) * (NT * TPW * PT);
  Cx* const tile2 = tile + (NT - 1) * TPW * PT;   // the second tile of a two-pass plan
  const Cx* __restrict__ tw1 = static_cast<const Cx*>(g.pass[R1 > 1 ? 1 : 0].tw);
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
      if constexpr (R1 == 1) {
        small_onepass<T, FWD, R, U, PT>(tile, t, one, nz, unit, sc);
      } else {
        Cx* const v = tile + t * PT;
        // the plan's two Stockham passes on the lane's own transform, one butterfly at a
        // time: pass 0 (radix R0, no twiddles) butterfly j reads elements j + r R1 of the
        // first tile and writes j R0 + r of the second; pass 1 (radix R1, ns = R0) butterfly
        // kk reads kk + r R0 of the second tile, with twiddle w_r(kk) at table entry
        // (r - 1) R0 + kk, and writes kk + r R0 of the first
        Cx* const v2 = tile2 + t * PT;
#pragma unroll 1
        for (int j = 0; j < R1; ++j) {
          T x[2 * R0], y[2 * R0];
#pragma unroll
          for (int r = 0; r < R0; ++r) {
            const Cx a = v[j + r * R1];
            x[2 * r] = a.x;
            x[2 * r + 1] = a.y;
          }
          P::template Bfly<FWD, R0, false>::run(x, y, one, nz);
#pragma unroll
          for (int r = 0; r < R0; ++r) v2[j * R0 + r] = P::mk(y[2 * r], y[2 * r + 1]);
        }
#pragma unroll 1
        for (int kk = 0; kk < R0; ++kk) {
          T x[4 * R1 - 2], y[2 * R1];
#pragma unroll
          for (int r = 0; r < R1; ++r) {
            const Cx a = v2[kk + r * R0];
            x[2 * r] = a.x;
            x[2 * r + 1] = a.y;
          }
#pragma unroll
          for (int r = 1; r < R1; ++r) {
            const Cx w = __ldg(tw1 + (r - 1) * R0 + kk);
            x[2 * R1 + 2 * (r - 1)] = w.x;
            x[2 * R1 + 2 * (r - 1) + 1] = w.y;
          }
          P::template Bfly<FWD, R1, true>::run(x, y, one, nz);
#pragma unroll
          for (int r = 0; r < R1; ++r)
            v[kk + r * R0] = unit ? P::mk(y[2 * r], y[2 * r + 1])
                                  : P::mk(P::mul(y[2 * r], sc), P::mul(y[2 * r + 1], sc));
        }
      }
    }
    __syncwarp();
    small_store<R, U, PT, K>(tile, dst, nt, lane, out_packed, out_rfast, ol, oe);
    __syncwarp();   // the tile is refilled by the warp's next chunk
  }
}

// Pipelined variant of the one-pass kernel: the warp's chunks are staged by asynchronous
// copies (cp.async, no registers held) into two tiles in turn, so that the next chunk is in
// flight while the current one is computed and stored; chunks of half the size keep the
// shared memory per warp.
__device__ __forceinline__ void small_cp_async(void* dst, const void* src, int bytes) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  if (bytes == 16)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(d), "l"(src) : "memory");
}

template <class T, bool FWD, int R>
__global__ void __launch_bounds__(kSmallThreads,
                                  (sizeof(T) == 8 && R <= 8) ? 3 : (sizeof(T) == 8 && R == 16) ? 1 : 2)
small_kernel_pipe(const GroupDesc g, const typename Prec<T>::C* in, typename Prec<T>::C* out) {
  using P = Prec<T>;
  using Cx = typename P::C;
  constexpr int KF = small_k(R, (int)sizeof(Cx));
  constexpr int K = KF > 1 ? KF / 2 : 1, TPW = 32 * K, PT = small_pitch(R, (int)sizeof(Cx));
  constexpr int U = 128 / (int)sizeof(Cx);
  extern __shared__ double2 small_smem[];
  const int lane = threadIdx.x & 31;
  Cx* const tiles = reinterpret_cast<Cx*>(small_smem) + (threadIdx.x >> 5) * (2 * TPW * PT);
  const int64_t ntr = g.total_sub;
  const int64_t nchunks = (ntr + TPW - 1) / TPW;
  const int64_t wstride = (int64_t)gridDim.x * kSmallWarps;
  const int64_t il = g.in_line, ie = g.in_elem, ol = g.out_line, oe = g.out_elem;
  const bool in_rfast = ie == 1, out_rfast = oe == 1;
  const bool in_packed = in_rfast && il == R, out_packed = out_rfast && ol == R;
  const bool unit = g.unit_scale != 0;
  const T sc = sizeof(T) == 4 ? (T)g.scale_f32 : (T)g.scale;
  T one, nz;
  P::units(one, nz);
  auto issue = [&](int64_t ch, Cx* tile) {
    const int64_t t0 = ch * TPW;
    const int nt = (int)min((int64_t)TPW, ntr - t0);
    const Cx* src = in + t0 * il;
    if (in_packed) {
#pragma unroll
      for (int k = 0; k < R * K; ++k) {
        const int e = k * 32 + lane;
        if (e < nt * R)
          small_cp_async(tile + (e / R) * PT + small_slot<R, U>(e / R, e % R), src + e, (int)sizeof(Cx));
      }
    } else {
#pragma unroll
      for (int k = 0; k < R * K; ++k) {
        const int e = k * 32 + lane;
        const int t = in_rfast ? e / R : e % TPW;
        const int r = in_rfast ? e - t * R : e / TPW;
        if (t < nt)
          small_cp_async(tile + t * PT + small_slot<R, U>(t, r), src + (int64_t)t * il + (int64_t)r * ie,
                         (int)sizeof(Cx));
      }
    }
  };
  int64_t ch = (int64_t)blockIdx.x * kSmallWarps + (threadIdx.x >> 5);
  int b = 0;
  if (ch < nchunks) issue(ch, tiles);
  asm volatile("cp.async.commit_group;" ::: "memory");
  for (; ch < nchunks; ch += wstride) {
    Cx* const tile = tiles + b * (TPW * PT);
    if (ch + wstride < nchunks) issue(ch + wstride, tiles + (b ^ 1) * (TPW * PT));
    asm volatile("cp.async.commit_group;" ::: "memory");
    asm volatile("cp.async.wait_group 1;" ::: "memory");   // this chunk's copies have landed
    __syncwarp();
    const int64_t t0 = ch * TPW;
    const int nt = (int)min((int64_t)TPW, ntr - t0);
#pragma unroll 1
    for (int k = 0; k < K; ++k) small_onepass<T, FWD, R, U, PT>(tile, k * 32 + lane, one, nz, unit, sc);
    __syncwarp();
    small_store<R, U, PT, K>(tile, out + t0 * ol, nt, lane, out_packed, out_rfast, ol, oe);
    __syncwarp();   // this tile is refilled by the chunk after next
    b ^= 1;
  }
  asm volatile("cp.async.wait_group 0;" ::: "memory");
}

template <class T>
size_t small_smem(int R, int tiles) {
  constexpr int es = (int)sizeof(typename Prec<T>::C);
  return (size_t)kSmallWarps * tiles * 32 * small_k(R, es) * small_pitch(R, es) * es;
}

// Two-pass binary32 plans with a compiled variant: the planner's radix pairs for the
// 13-smooth sizes 18 .. 32
constexpr int kSmallPairs[][2] = {{6, 3}, {10, 2}, {7, 3}, {11, 2}, {12, 2}, {5, 5},
                                  {13, 2}, {9, 3}, {14, 2}, {15, 2}, {16, 2}};

template <class T, bool FWD>
const void* small_fn(int R0, int R1) {
  if (R1 == 1) {
    switch (R0) {
#define LFG_SMALL_CASE(RR) \
  case RR: return (const void*)small_kernel<T, FWD, RR, 1>;
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
  if constexpr (sizeof(T) == 4) {
#define LFG_SMALL_PAIR(A, B) \
  if (R0 == A && R1 == B) return (const void*)small_kernel<T, FWD, A, B>;
    LFG_SMALL_PAIR(6, 3)
    LFG_SMALL_PAIR(10, 2)
    LFG_SMALL_PAIR(7, 3)
    LFG_SMALL_PAIR(11, 2)
    LFG_SMALL_PAIR(12, 2)
    LFG_SMALL_PAIR(5, 5)
    LFG_SMALL_PAIR(13, 2)
    LFG_SMALL_PAIR(9, 3)
    LFG_SMALL_PAIR(14, 2)
    LFG_SMALL_PAIR(15, 2)
    LFG_SMALL_PAIR(16, 2)
#undef LFG_SMALL_PAIR
  }
  return nullptr;
}

const void* small_kernel_fn(int precision, bool fwd, int R0, int R1) {
  if (precision == 0) return fwd ? small_fn<double, true>(R0, R1) : small_fn<double, false>(R0, R1);
  return fwd ? small_fn<float, true>(R0, R1) : small_fn<float, false>(R0, R1);
}

size_t small_smem_bytes(int precision, int R0, int R1) {
  const int tiles = R1 > 1 ? 2 : 1;
  return precision == 0 ? small_smem<double>(R0 * R1, tiles) : small_smem<float>(R0 * R1, tiles);
}

// One-pass plans run the pipelined variant (1 GiB batches on GB300: binary32 0.90-0.93 of HBM
// against 0.80-0.91, binary64 N = 2 .. 12 and 16 up to 11 % faster), except binary64 R = 13 ..
// 15, which measured 5-7 % slower pipelined; LFG_SMALL_PIPE=0 in the environment turns it off
// (for comparisons; the same bits).
bool small_pipe(int precision, int r0, int r1) {
  if (r1 > 1 || (precision == 0 && r0 >= 13 && r0 <= 15)) return false;
  const char* s = std::getenv("LFG_SMALL_PIPE");
  return !(s && s[0] == '0');
}

size_t small_pipe_smem_bytes(int precision, int R) {
  const int es = precision == 0 ? 16 : 8;
  const int kf = small_k(R, es), k = kf > 1 ? kf / 2 : 1;
  return (size_t)kSmallWarps * 2 * 32 * k * small_pitch(R, es) * es;
}

const void* small_pipe_fn(int precision, bool fwd, int R) {
  switch (R * 4 + precision * 2 + (fwd ? 1 : 0)) {
#define LFG_PIPE_CASE(RR)                                                   \
  case RR * 4 + 0: return (const void*)small_kernel_pipe<double, false, RR>; \
  case RR * 4 + 1: return (const void*)small_kernel_pipe<double, true, RR>;  \
  case RR * 4 + 2: return (const void*)small_kernel_pipe<float, false, RR>;  \
  case RR * 4 + 3: return (const void*)small_kernel_pipe<float, true, RR>;
    LFG_PIPE_CASE(2)
    LFG_PIPE_CASE(3)
    LFG_PIPE_CASE(4)
    LFG_PIPE_CASE(5)
    LFG_PIPE_CASE(6)
    LFG_PIPE_CASE(7)
    LFG_PIPE_CASE(8)
    LFG_PIPE_CASE(9)
    LFG_PIPE_CASE(10)
    LFG_PIPE_CASE(11)
    LFG_PIPE_CASE(12)
    LFG_PIPE_CASE(13)
    LFG_PIPE_CASE(14)
    LFG_PIPE_CASE(15)
    LFG_PIPE_CASE(16)
#undef LFG_PIPE_CASE
    default: return nullptr;
  }
}

// The radices of group g when the warp-tile kernel has a variant for its plan (r1 = 1: one
// pass), else false.
bool small_radices(const GroupDesc& g, int precision, int* r0, int* r1) {
  if (g.nsub != 1 || g.total_sub <= 0 || g.M < 2) return false;
  if (g.npass == 1 && g.M <= kSmallMaxN && g.pass[0].R == g.M && !g.pass[0].tw) {
    *r0 = g.M;
    *r1 = 1;
    return true;
  }
  const PassDesc &a = g.pass[0], &b = g.pass[1];
  if (g.npass == 2 && precision == 1 && g.M <= kSmallMaxTwoPassN && !a.tw && b.tw && !b.comp &&
      a.R * b.R == g.M && b.ns_loc == a.R && b.ns_g == a.R && small_kernel_fn(1, true, a.R, b.R)) {
    *r0 = a.R;
    *r1 = b.R;
    return true;
  }
  return false;
}

}  // namespace

bool small_kernel_applies(const GroupDesc& g, int precision) {
  int r0 = 0, r1 = 0;
  return small_radices(g, precision, &r0, &r1);
}

cudaError_t prepare_small_kernels() {
  for (int prec = 0; prec < 2; ++prec)
    for (int fwd = 0; fwd < 2; ++fwd) {
      auto allow = [&](int r0, int r1) -> cudaError_t {
        const void* fn = small_kernel_fn(prec, fwd != 0, r0, r1);
        const size_t s = small_smem_bytes(prec, r0, r1);
        if (!fn || s <= 48 * 1024) return cudaSuccess;
        return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s);
      };
      for (int R = 2; R <= kSmallMaxN; ++R) {
        if (cudaError_t e = allow(R, 1)) return e;
        const size_t sp = small_pipe_smem_bytes(prec, R);
        if (sp > 48 * 1024)
          if (cudaError_t e = cudaFuncSetAttribute(small_pipe_fn(prec, fwd != 0, R),
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sp))
            return e;
      }
      for (const auto& pr : kSmallPairs)
        if (cudaError_t e = allow(pr[0], pr[1])) return e;
    }
  return cudaSuccess;
}

unsigned small_grid(const GroupDesc& g, int precision) {
  int r0 = 0, r1 = 0;
  if (!small_radices(g, precision, &r0, &r1)) return 0;
  const int R = g.M;
  const bool pipe = small_pipe(precision, r0, r1);
  const void* fn = pipe ? small_pipe_fn(precision, true, R) : small_kernel_fn(precision, true, r0, r1);
  const size_t smem = pipe ? small_pipe_smem_bytes(precision, R) : small_smem_bytes(precision, r0, r1);
  int dev = 0, sms = 1, per_sm = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kSmallThreads, smem) != cudaSuccess ||
      per_sm < 1)
    per_sm = 1;
  const int kf = small_k(R, precision == 0 ? 16 : 8);
  const int64_t tpb = (int64_t)kSmallWarps * 32 * (pipe ? (kf > 1 ? kf / 2 : 1) : kf);
  const int64_t need = (g.total_sub + tpb - 1) / tpb;
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(need, (int64_t)sms * per_sm));
}

cudaError_t launch_small(const GroupDesc& gd, int precision, bool fwd, const void* in, void* out,
                         unsigned grid, cudaStream_t stream) {
  int r0 = 0, r1 = 0;
  if (!small_radices(gd, precision, &r0, &r1)) return cudaErrorInvalidValue;
  GroupDesc g = gd;
  set_divisors(g);
  const bool pipe = small_pipe(precision, r0, r1);
  const size_t smem = pipe ? small_pipe_smem_bytes(precision, g.M) : small_smem_bytes(precision, r0, r1);
  void* args[] = {(void*)&g, (void*)&in, (void*)&out};
  return cudaLaunchKernel(pipe ? small_pipe_fn(precision, fwd, g.M) : small_kernel_fn(precision, fwd, r0, r1),
                          dim3(grid), dim3(kSmallThreads), args, smem, stream);
}

}  // namespace lfg
