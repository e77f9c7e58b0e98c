// Binary32 groups of two-group power-of-two plans over contiguous lines, staged through
// registers instead of copy loops.
//
// A two-group plan of N = P * Q points runs its first passes as Q sub-problems of P points
// (sub-problem b reads x[b + Q i], writes the row z[b P + m]) and its last passes as P
// sub-problems of Q points (sub-problem m reads the column z[i P + m], writes the column
// out[o P + m]).  Each CTA here takes one tile of C neighbouring sub-problems (4096 points,
// 16 per thread) and runs the group's two passes:
// * the first pass loads its butterflies' inputs straight from global memory into registers,
//   neighbouring threads on neighbouring sub-problems (runs of C contiguous elements), and
//   writes its outputs to one shared-memory tile (odd pitch: conflict-free across
//   sub-problems);
// * after one barrier the second pass reads the tile and stores its outputs straight to
//   global memory: along the row (neighbouring threads on neighbouring outputs) for a first
//   group, across sub-problems (runs of C) for a second group.
// No element passes through a copy loop, and there is one barrier per tile.  Latency is
// hidden by occupancy (several CTAs per SM) and by the sixteen independent loads of each
// thread's first butterfly.
//
// The butterflies perform the same operations on the same operands as every other binary32
// kernel of the library (the generated codelets, the same twiddle values and compensated
// products), so the bits are the same.  The second group's twiddle tables are kept in pass
// order (index k P + m: the sub-problem index fastest), which neighbouring threads read as
// contiguous runs.
#include <cuda_runtime.h>

#include "kernels.h"
#include "stockham_dev.cuh"

namespace lfg {
using namespace dev;
namespace {

constexpr int kDirectThreads = 256;
constexpr int kDirectPoints = 4096;   // points per tile

enum DirectTarget { kToTile = 0, kToRows = 1, kToCols = 2 };

// One pass of a group with compile-time geometry: sub-problems of M points, tile of C
// sub-problems at pitch PM, radix R, NSL = product of the group's earlier radices, NSUB = the
// other group's size; TWSUB: a second group (twiddle index k * NSUB + m); MODE 0 untwiddled,
// 1 twiddled, 2 compensated (hi, lo) twiddles.  FROM_GLOBAL: inputs from the tile's first
// column element `gin` (element (c, i) at gin[c + i NSUB]), else from the shared tile.
template <bool FWD, int M, int C, int R, int NSL, int NSUB, bool TWSUB, int MODE, bool FROM_GLOBAL,
          int TO>
__device__ __forceinline__ void direct_pass(const float2* __restrict__ gin, const float2* src,
                                            float2* dst, float2* __restrict__ gout,
                                            const float2* __restrict__ tw, int sub0, bool unit,
                                            float sc) {
  using P = Prec<float>;
  constexpr int PM = sub_pitch(M) | 1;
  constexpr int MR = M / R;
  constexpr int NB = C * MR;
  constexpr int NSG = TWSUB ? NSUB * NSL : NSL;
  constexpr bool TW = MODE == 1;
  constexpr bool JFAST = TO == kToRows;   // row stores: neighbouring threads along the row
  static_assert(NB % kDirectThreads == 0, "whole butterflies per thread");
  const float one = 1.0f, nz = -0.0f;   // (the binary32 codelets do not use them)
#pragma unroll
  for (int it = 0; it < NB / kDirectThreads; ++it) {
    const int q = (int)threadIdx.x + it * kDirectThreads;
    const int c = JFAST ? q / MR : q % C;
    const int j = JFAST ? q % MR : q / C;
    float x[TW ? 4 * R - 2 : 2 * R];
    float y[2 * R];
    if (FROM_GLOBAL) {
      const float2* s = gin + c + j * NSUB;
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const float2 v = s[r * MR * NSUB];
        x[2 * r] = v.x;
        x[2 * r + 1] = v.y;
      }
    } else if (MR % 16 == 0) {
      const float2* s = src + c * PM + spad(j);
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const float2 v = s[r * (MR + MR / 16)];
        x[2 * r] = v.x;
        x[2 * r + 1] = v.y;
      }
    } else {
      const float2* s = src + c * PM;
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const float2 v = s[spad(j + r * MR)];
        x[2 * r] = v.x;
        x[2 * r + 1] = v.y;
      }
    }
    const int b = j / NSL;
    const int k = j % NSL;
    const int kg = TWSUB ? k * NSUB + sub0 + c : k;
    if (MODE == 1) {
      const float2* __restrict__ w = tw + kg;
#pragma unroll
      for (int r = 0; r < R - 1; ++r) {
        const float2 v = __ldg(w + r * NSG);
        x[2 * R + 2 * r] = v.x;
        x[2 * R + 2 * r + 1] = v.y;
      }
    } else if (MODE == 2) {
      const float2* __restrict__ wh = tw + kg;
      const float2* __restrict__ wl = wh + (R - 1) * NSG;
#pragma unroll
      for (int r = 1; r < R; ++r) {
        const float2 h = __ldg(wh + (r - 1) * NSG), l = __ldg(wl + (r - 1) * NSG);
        const float wrh = h.x, wih = h.y, wrl = l.x, wil = l.y;
        const float a = x[2 * r], bi = x[2 * r + 1];
        const float cr = P::fma(a, wrl, -P::mul(bi, wil));
        const float ci = P::fma(a, wil, P::mul(bi, wrl));
        x[2 * r] = P::fma(a, wrh, P::fma(-bi, wih, cr));
        x[2 * r + 1] = P::fma(a, wih, P::fma(bi, wrh, ci));
      }
    }
    BflyF<FWD, R, TW>::run(x, y, one, nz);
    const int d0 = b * NSL * R + k;
    if (TO == kToTile) {
      float2* o = dst + c * PM;
      if (NSL % 16 == 0) {
#pragma unroll
        for (int r = 0; r < R; ++r) o[spad(d0) + r * (NSL + NSL / 16)] = make_float2(y[2 * r], y[2 * r + 1]);
      } else {
#pragma unroll
        for (int r = 0; r < R; ++r) o[spad(d0 + r * NSL)] = make_float2(y[2 * r], y[2 * r + 1]);
      }
    } else {
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const float2 v = unit ? make_float2(y[2 * r], y[2 * r + 1])
                              : make_float2(__fmul_rn(y[2 * r], sc), __fmul_rn(y[2 * r + 1], sc));
        if (TO == kToRows) gout[c * M + d0 + r * NSL] = v;
        else gout[c + (d0 + r * NSL) * NSUB] = v;
      }
    }
  }
}

// A two-pass group (radices R0, R1) of M points with the other group's size NSUB.
template <bool FWD, int M, int NSUB, bool TWSUB, bool COMP, int R0, int R1>
__global__ void __launch_bounds__(kDirectThreads, 3)
direct_kernel_f32(const GroupDesc g, const float2* in, float2* out) {
  constexpr int C = kDirectPoints / M;
  constexpr int PM = sub_pitch(M) | 1;
  constexpr int MODE_T = TWSUB ? (COMP ? 2 : 1) : 1;
  static_assert(M == R0 * R1 && NSUB % C == 0, "tile geometry");
  __shared__ float2 tile[C * PM];
  const int64_t s0 = (int64_t)blockIdx.x * C;
  const int64_t line = s0 / NSUB;
  const int sub0 = (int)(s0 - line * NSUB);
  const float2* gin = in + line * g.in_line + sub0;
  float2* gout = out + line * g.out_line + (TWSUB ? (int64_t)sub0 : (int64_t)sub0 * M);
  direct_pass<FWD, M, C, R0, 1, NSUB, TWSUB, TWSUB ? MODE_T : 0, true, kToTile>(
      gin, nullptr, tile, nullptr, static_cast<const float2*>(g.pass[0].tw), sub0, true, 1.0f);
  __syncthreads();
  direct_pass<FWD, M, C, R1, R0, NSUB, TWSUB, MODE_T, false, TWSUB ? kToCols : kToRows>(
      nullptr, tile, nullptr, gout, static_cast<const float2*>(g.pass[1].tw), sub0,
      g.unit_scale != 0, g.scale_f32);
}

// The groups with a kernel here: M, the other group's size, second group, compensated
// twiddles, radices.  They are the groups of the planner's binary32 plans of 2^14 (16.8 | 16.8),
// 2^15 (16.16 | 16.8) and 2^16 (16.16 | 16.16, with or without compensation).
struct DirectGroup {
  int M, nsub, twsub, comp, r0, r1;
};
constexpr DirectGroup kDirectGroups[] = {
    {128, 128, 0, 0, 16, 8},  {128, 128, 1, 0, 16, 8},  {256, 128, 0, 0, 16, 16},
    {128, 256, 1, 0, 16, 8},  {256, 256, 0, 0, 16, 16}, {256, 256, 1, 1, 16, 16},
    {256, 256, 1, 0, 16, 16}};
constexpr int kDirectVariants = (int)(sizeof(kDirectGroups) / sizeof(kDirectGroups[0]));

using DirectFn = void (*)(const GroupDesc, const float2*, float2*);

template <bool FWD>
DirectFn direct_fn(int v) {
  switch (v) {
    case 0: return direct_kernel_f32<FWD, 128, 128, false, false, 16, 8>;
    case 1: return direct_kernel_f32<FWD, 128, 128, true, false, 16, 8>;
    case 2: return direct_kernel_f32<FWD, 256, 128, false, false, 16, 16>;
    case 3: return direct_kernel_f32<FWD, 128, 256, true, false, 16, 8>;
    case 4: return direct_kernel_f32<FWD, 256, 256, false, false, 16, 16>;
    case 5: return direct_kernel_f32<FWD, 256, 256, true, true, 16, 16>;
    case 6: return direct_kernel_f32<FWD, 256, 256, true, false, 16, 16>;
    default: return nullptr;
  }
}

}  // namespace

int direct_variant_f32(int M, int nsub, bool twsub, bool comp, const int* radices, int npass) {
  if (npass != 2) return -1;
  for (int v = 0; v < kDirectVariants; ++v) {
    const DirectGroup& d = kDirectGroups[v];
    if (d.M == M && d.nsub == nsub && (d.twsub != 0) == twsub && (d.comp != 0) == comp &&
        d.r0 == radices[0] && d.r1 == radices[1])
      return v;
  }
  return -1;
}

cudaError_t launch_direct_f32(const GroupDesc& gd, bool fwd, const void* in, void* out,
                              int variant, cudaStream_t stream) {
  if (variant < 0 || variant >= kDirectVariants) return cudaErrorInvalidValue;
  const DirectGroup& d = kDirectGroups[variant];
  GroupDesc g = gd;
  set_divisors(g);
  const int C = kDirectPoints / d.M;
  // the layout the kernel is compiled for: columns in, rows (first group) or columns out
  const bool ok = g.M == d.M && g.nsub == d.nsub && g.npass == 2 && g.in_sub == 1 &&
                  g.in_elem == d.nsub && (g.twsub != 0) == (d.twsub != 0) &&
                  (d.twsub ? (g.out_sub == 1 && g.out_elem == d.nsub)
                           : (g.out_sub == d.M && g.out_elem == 1)) &&
                  g.total_sub % C == 0;
  if (!ok) return cudaErrorInvalidValue;
  const int64_t ntiles = g.total_sub / C;
  if (ntiles == 0) return cudaSuccess;
  if (ntiles > 0x7fffffff) return cudaErrorInvalidValue;
  const DirectFn kern = fwd ? direct_fn<true>(variant) : direct_fn<false>(variant);
  kern<<<(unsigned)ntiles, kDirectThreads, 0, stream>>>(g, static_cast<const float2*>(in),
                                                        static_cast<float2*>(out));
  return cudaGetLastError();
}

}  // namespace lfg
