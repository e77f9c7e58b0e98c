// Device helpers of the register-staged binary32 kernels (direct_f32.cu, and the rows of
// binary32 r2c plans in real.cu): tile geometry and one pass whose inputs come from global
// memory or a shared tile and whose outputs go to a shared tile or global memory.
#pragma once
#include <cuda_runtime.h>

#include "kernels.h"
#include "stockham_dev.cuh"

namespace lfg {
namespace dfx {
using namespace dev;

// Global layouts of a group's sub-problems (element i of sub-problem c of the tile):
//   kFirstOfTwo   in c + i NSUB (columns), out c M + i (rows)
//   kSecondOfTwo  in columns, out c + i NSUB (columns)
//   kSingle       in c LDI + i, out c LDO + i (rows at the plan's line distances)
constexpr int kFirstOfTwo = kDirectFirstOfTwo;
constexpr int kSecondOfTwo = kDirectSecondOfTwo;
constexpr int kSingle = kDirectSingle;

constexpr int kDirectPoints = 4096;   // points per tile (16 per thread)


// *RT: the calling thread's own sub-problem at run-time addresses (`tin` / `tout`, element
// stride `tstride`), for layouts whose sub-problems are not evenly spaced (the columns of a
// batch of images, rows at a line list); the thread's sub-problem must stay fixed over the
// pass (across sub-problems with T a multiple of C, or one butterfly per thread along them).
enum DirectSrc { kFromTile = 0, kFromCols = 1, kFromRows = 2, kFromColsRT = 3, kFromRowsRT = 4 };
enum DirectDst { kToTile = 0, kToRows = 1, kToCols = 2, kToColsRT = 3 };

// Tile pitch: odd for tiles of 16 or more sub-problems, 2 mod 16 for 8 (a half-warp then
// spans 8 sub-problems and two neighbouring elements), the padded length otherwise (those
// passes walk along the sub-problem).
// Sub-problems per tile and threads per CTA: 4096-point tiles, except the 512-point groups of
// two-group plans, whose tiles of 16 columns (128-byte runs) hold 8192 points on 512 threads.
LFG_HD constexpr int direct_width(int layout, int M) {
  return layout != kDirectSingle && M == 512 ? 16 : kDirectPoints / M;
}
LFG_HD constexpr int direct_threads(int layout, int M) { return direct_width(layout, M) * M / 16; }

LFG_HD constexpr int direct_pitch(int M, int C) {
  return C >= 16 ? (sub_pitch(M) | 1) : (C == 8 ? sub_pitch(M) + ((2 - sub_pitch(M)) & 15) : sub_pitch(M));
}

// One pass with compile-time geometry: sub-problems of M points, tile of C sub-problems at
// pitch PM, radix R, NSL = product of the group's earlier radices, NSUB = the other group's
// size; TWSUB: a second group (twiddle index k * NSUB + m); MODE 0 untwiddled, 1 twiddled,
// 2 compensated (hi, lo) twiddles.  `gin` / `gout`: the tile's first element in global
// memory; ldi / ldo: line distances of rows; count: sub-problems of the tile present (rows
// only; the others are never loaded or stored).
template <bool FWD, int M, int C, int PM, int T, int R, int NSL, int NSUB, bool TWSUB, int MODE,
          int SRC, int DST>
__device__ __forceinline__ void direct_pass(const float2* __restrict__ gin, int64_t ldi,
                                            const float2* src, float2* dst,
                                            float2* __restrict__ gout, int64_t ldo,
                                            const float2* __restrict__ tw, int sub0, int count,
                                            bool unit, float sc,
                                            const float2* __restrict__ tin = nullptr,
                                            float2* __restrict__ tout = nullptr,
                                            int64_t tstride = 0, bool tvalid = true) {
  using P = Prec<float>;
  constexpr int MR = M / R;
  constexpr int NB = C * MR;
  constexpr int NSG = TWSUB ? NSUB * NSL : NSL;
  constexpr bool TW = MODE == 1;
  // across sub-problems where a column is read or written and for a second group's passes
  // (its twiddles are contiguous across sub-problems), along them where a row is
  constexpr bool CFAST = (SRC == kFromCols || DST == kToCols || SRC == kFromColsRT ||
                          DST == kToColsRT || TWSUB) &&
                         SRC != kFromRows && SRC != kFromRowsRT && DST != kToRows;
  static_assert(NB % T == 0, "whole butterflies per thread");
  static_assert(!(SRC == kFromColsRT || SRC == kFromRowsRT || DST == kToColsRT) ||
                    (CFAST ? T % C == 0 : NB == T),
                "a thread's own sub-problem stays fixed over the pass");
  const float one = 1.0f, nz = -0.0f;   // (the binary32 codelets do not use them)
#pragma unroll
  for (int it = 0; it < NB / T; ++it) {
    const int q = (int)threadIdx.x + it * T;
    const int c = CFAST ? q % C : q / MR;
    const int j = CFAST ? q / C : q % MR;
    float x[TW ? 4 * R - 2 : 2 * R];
    float y[2 * R];
    if (SRC == kFromCols) {
      const float2* s = gin + c + j * NSUB;
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const float2 v = s[r * MR * NSUB];
        x[2 * r] = v.x;
        x[2 * r + 1] = v.y;
      }
    } else if (SRC == kFromRows) {
      const float2* s = gin + c * ldi + j;
      const bool present = c < count;
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const float2 v = present ? s[r * MR] : make_float2(0.0f, 0.0f);
        x[2 * r] = v.x;
        x[2 * r + 1] = v.y;
      }
    } else if (SRC == kFromColsRT) {
      const float2* s = tin + (int64_t)j * tstride;
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const float2 v = tvalid ? s[(int64_t)r * MR * tstride] : make_float2(0.0f, 0.0f);
        x[2 * r] = v.x;
        x[2 * r + 1] = v.y;
      }
    } else if (SRC == kFromRowsRT) {
      const float2* s = tin + j;
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const float2 v = tvalid ? s[r * MR] : make_float2(0.0f, 0.0f);
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
      // (hi re, hi im, lo re, lo im) per twiddle
      const float4* __restrict__ w4 = reinterpret_cast<const float4*>(tw) + kg;
#pragma unroll
      for (int r = 1; r < R; ++r) {
        const float4 q4 = __ldg(w4 + (r - 1) * NSG);
        const float wrh = q4.x, wih = q4.y, wrl = q4.z, wil = q4.w;
        const float a = x[2 * r], bi = x[2 * r + 1];
        const float cr = P::fma(a, wrl, -P::mul(bi, wil));
        const float ci = P::fma(a, wil, P::mul(bi, wrl));
        x[2 * r] = P::fma(a, wrh, P::fma(-bi, wih, cr));
        x[2 * r + 1] = P::fma(a, wih, P::fma(bi, wrh, ci));
      }
    }
    BflyF<FWD, R, TW>::run(x, y, one, nz);
    const int d0 = b * NSL * R + k;
    if (DST == kToTile) {
      float2* o = dst + c * PM;
      if (NSL % 16 == 0) {
#pragma unroll
        for (int r = 0; r < R; ++r) o[spad(d0) + r * (NSL + NSL / 16)] = make_float2(y[2 * r], y[2 * r + 1]);
      } else {
#pragma unroll
        for (int r = 0; r < R; ++r) o[spad(d0 + r * NSL)] = make_float2(y[2 * r], y[2 * r + 1]);
      }
    } else if (DST == kToColsRT) {
      if (tvalid) {
#pragma unroll
        for (int r = 0; r < R; ++r) {
          const float2 v = unit ? make_float2(y[2 * r], y[2 * r + 1])
                                : make_float2(__fmul_rn(y[2 * r], sc), __fmul_rn(y[2 * r + 1], sc));
          tout[(int64_t)(d0 + r * NSL) * tstride] = v;
        }
      }
    } else if (DST == kToCols || c < count) {
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const float2 v = unit ? make_float2(y[2 * r], y[2 * r + 1])
                              : make_float2(__fmul_rn(y[2 * r], sc), __fmul_rn(y[2 * r + 1], sc));
        if (DST == kToRows) gout[c * ldo + d0 + r * NSL] = v;
        else gout[c + (d0 + r * NSL) * NSUB] = v;
      }
    }
  }
}


}  // namespace dfx
}  // namespace lfg
