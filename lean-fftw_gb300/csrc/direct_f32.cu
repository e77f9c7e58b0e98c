// Binary32 groups over contiguous lines, staged through registers instead of copy loops.
//
// A two-group plan of N = P * Q points runs its first passes as Q sub-problems of P points
// (sub-problem b reads x[b + Q i], writes the row z[b P + m]) and its last passes as P
// sub-problems of Q points (sub-problem m reads the column z[i P + m], writes the column
// out[o P + m]); a one-group plan runs whole lines (rows in, rows out).  Each CTA here takes
// one tile of C neighbouring sub-problems (4096 points, 16 per thread) and runs the group's
// two or three passes:
// * the first pass loads its butterflies' inputs straight from global memory into registers
//   -- neighbouring threads on neighbouring sub-problems for columns (runs of C contiguous
//   elements), on neighbouring elements for rows -- and writes its outputs to a shared tile;
// * a middle pass goes from one shared tile to the other;
// * the last pass reads a shared tile and stores its outputs straight to global memory:
//   along the row (neighbouring threads on neighbouring outputs) or across sub-problems.
// No element passes through a copy loop, and there is one barrier per pass boundary.  The
// tile pitch is chosen per tile width so that the passes that walk across sub-problems hit
// distinct banks.  Latency is hidden by occupancy (three CTAs per SM) and by the independent
// loads of each thread's first butterflies.
//
// The butterflies perform the same operations on the same operands as every other binary32
// kernel of the library (the generated codelets, the same twiddle values and compensated
// products), so the bits are the same.  A second group's twiddle tables are kept in pass
// order (index k P + m: the sub-problem index fastest), which neighbouring threads read as
// contiguous runs, and a compensated twiddle as one (hi, lo) quadruple (one 16-byte load).
#include <cuda_runtime.h>

#include "direct_dev.cuh"
#include "kernels.h"

namespace lfg {
using namespace dev;
namespace {
using namespace dfx;

// A group of two or three passes (radices R0, R1, R2; R2 = 0: two) of M points; NSUB = the
// other group's size (two-group layouts).
template <bool FWD, int LAYOUT, int M, int NSUB, bool COMP, int R0, int R1, int R2>
__global__ void __launch_bounds__(direct_threads(LAYOUT, M), direct_threads(LAYOUT, M) > 256 ? 1 : 3)
direct_kernel_f32(const GroupDesc g, const float2* in, float2* out) {
  constexpr bool TWSUB = LAYOUT == kSecondOfTwo;
  constexpr int C = direct_width(LAYOUT, M);
  constexpr int T = direct_threads(LAYOUT, M);
  constexpr int PM = direct_pitch(M, C);
  constexpr int MODE_T = TWSUB ? (COMP ? 2 : 1) : 1;
  constexpr int SRC0 = LAYOUT == kSingle ? kFromRows : kFromCols;
  constexpr int DSTL = LAYOUT == kSecondOfTwo ? kToCols : kToRows;
  static_assert(M == R0 * R1 * (R2 > 0 ? R2 : 1) && C >= 1, "tile geometry");
  extern __shared__ float2 smem_direct[];
  float2* A = smem_direct;
  float2* B = smem_direct + C * PM;
  const int64_t s0 = (int64_t)blockIdx.x * C;
  int sub0 = 0, count = C;
  const float2* gin;
  float2* gout;
  int64_t ldi = M, ldo = M;
  if (LAYOUT == kSingle) {
    count = (int)min((int64_t)C, g.total_sub - s0);
    gin = in + s0 * g.in_line;
    gout = out + s0 * g.out_line;
    ldi = g.in_line;
    ldo = g.out_line;
  } else {
    const int64_t line = s0 / NSUB;
    sub0 = (int)(s0 - line * NSUB);
    gin = in + line * g.in_line + sub0;
    gout = out + line * g.out_line + (TWSUB ? (int64_t)sub0 : (int64_t)sub0 * M);
  }
  const bool unit = g.unit_scale != 0;
  const float sc = g.scale_f32;
  const float2* tw0 = static_cast<const float2*>(g.pass[0].tw);
  const float2* tw1 = static_cast<const float2*>(g.pass[1].tw);
  direct_pass<FWD, M, C, PM, T, R0, 1, NSUB, TWSUB, TWSUB ? MODE_T : 0, SRC0, kToTile>(
      gin, ldi, nullptr, A, nullptr, 0, tw0, sub0, count, true, 1.0f);
  __syncthreads();
  if constexpr (R2 > 0) {
    direct_pass<FWD, M, C, PM, T, R1, R0, NSUB, TWSUB, MODE_T, kFromTile, kToTile>(
        nullptr, 0, A, B, nullptr, 0, tw1, sub0, count, true, 1.0f);
    __syncthreads();
    direct_pass<FWD, M, C, PM, T, R2, R0 * R1, NSUB, TWSUB, MODE_T, kFromTile, DSTL>(
        nullptr, 0, B, nullptr, gout, ldo, static_cast<const float2*>(g.pass[2].tw), sub0,
        count, unit, sc);
  } else {
    direct_pass<FWD, M, C, PM, T, R1, R0, NSUB, TWSUB, MODE_T, kFromTile, DSTL>(
        nullptr, 0, A, nullptr, gout, ldo, tw1, sub0, count, unit, sc);
  }
}

using DirectFn = void (*)(const GroupDesc, const float2*, float2*);

// The columns of a batch of images (the first axis of a rank-2 plan): sub-problem s is column
// s mod nsub of image s / nsub, element i at line * line_dist + col * sub_stride + i * elem
// (input and output alike, their own strides).  A CTA of M threads takes 16 neighbouring
// sub-problems (a tile may straddle two images); each thread's column base is computed once,
// the first pass loads across the 16 columns (128-byte runs), the last pass stores likewise.
template <bool FWD, int M, int R0, int R1, int R2>
__global__ void __launch_bounds__(M, M > 256 ? 1 : 2)
direct_cols_kernel_f32(const GroupDesc g, const float2* in, float2* out) {
  constexpr int C = 16;
  constexpr int T = M;
  constexpr int PM = direct_pitch(M, C);
  static_assert(M == R0 * R1 * (R2 > 0 ? R2 : 1), "tile geometry");
  extern __shared__ float2 smem_direct[];
  float2* A = smem_direct;
  float2* B = smem_direct + C * PM;
  const int c = (int)threadIdx.x % C;   // the thread's column in the first and last passes
  const int64_t sidx = (int64_t)blockIdx.x * C + c;
  const bool valid = sidx < g.total_sub;
  const int64_t line = valid ? sidx / g.nsub : 0;
  const int64_t col = valid ? sidx - line * g.nsub : 0;
  const float2* tin = in + line * g.in_line + col * g.in_sub;
  float2* tout = out + line * g.out_line + col * g.out_sub;
  const bool unit = g.unit_scale != 0;
  const float sc = g.scale_f32;
  const float2* tw1 = static_cast<const float2*>(g.pass[1].tw);
  direct_pass<FWD, M, C, PM, T, R0, 1, 0, false, 0, kFromColsRT, kToTile>(
      nullptr, 0, nullptr, A, nullptr, 0, nullptr, 0, C, true, 1.0f, tin, nullptr, g.in_elem, valid);
  __syncthreads();
  if constexpr (R2 > 0) {
    direct_pass<FWD, M, C, PM, T, R1, R0, 0, false, 1, kFromTile, kToTile>(
        nullptr, 0, A, B, nullptr, 0, tw1, 0, C, true, 1.0f);
    __syncthreads();
    direct_pass<FWD, M, C, PM, T, R2, R0 * R1, 0, false, 1, kFromTile, kToColsRT>(
        nullptr, 0, B, nullptr, nullptr, 0, static_cast<const float2*>(g.pass[2].tw), 0, C, unit,
        sc, nullptr, tout, g.out_elem, valid);
  } else {
    direct_pass<FWD, M, C, PM, T, R1, R0, 0, false, 1, kFromTile, kToColsRT>(
        nullptr, 0, A, nullptr, nullptr, 0, tw1, 0, C, unit, sc, nullptr, tout, g.out_elem, valid);
  }
}

struct DirectCols {
  int M, r[3];
};
constexpr DirectCols kDirectCols[] = {
    {64, {16, 4, 0}}, {128, {16, 8, 0}}, {256, {16, 16, 0}}, {512, {16, 16, 2}}};
constexpr int kDirectColVariants = (int)(sizeof(kDirectCols) / sizeof(kDirectCols[0]));

template <bool FWD>
DirectFn direct_cols_fn(int v) {
  switch (v) {
    case 0: return direct_cols_kernel_f32<FWD, 64, 16, 4, 0>;
    case 1: return direct_cols_kernel_f32<FWD, 128, 16, 8, 0>;
    case 2: return direct_cols_kernel_f32<FWD, 256, 16, 16, 0>;
    case 3: return direct_cols_kernel_f32<FWD, 512, 16, 16, 2>;
    default: return nullptr;
  }
}

size_t direct_cols_smem(int v) {
  const DirectCols& d = kDirectCols[v];
  return (size_t)(d.r[2] > 0 ? 2 : 1) * 16 * direct_pitch(d.M, 16) * sizeof(float2);
}

// The groups with a kernel here: layout, M, the other group's size (1 for one group),
// compensated twiddles, radices.  They are the groups of the planner's binary32 plans of
// 2^9 .. 2^12 (one group) and 2^13 .. 2^18 (two groups: 16.8 | 16.4, 16.8 | 16.8,
// 16.16 | 16.8, 16.16 | 16.16, 16.16 | 2.16.16, 16.16.2 | 16.16.2; the second groups from
// 2^16 with and without compensation).
struct DirectGroup {
  int layout, M, nsub, comp, r[3];
};
constexpr DirectGroup kDirectGroups[] = {
    {kFirstOfTwo, 128, 128, 0, {16, 8, 0}},     {kSecondOfTwo, 128, 128, 0, {16, 8, 0}},
    {kFirstOfTwo, 256, 128, 0, {16, 16, 0}},    {kSecondOfTwo, 128, 256, 0, {16, 8, 0}},
    {kFirstOfTwo, 256, 256, 0, {16, 16, 0}},    {kSecondOfTwo, 256, 256, 1, {16, 16, 0}},
    {kSecondOfTwo, 256, 256, 0, {16, 16, 0}},   {kFirstOfTwo, 256, 512, 0, {16, 16, 0}},
    {kSecondOfTwo, 512, 256, 1, {2, 16, 16}},   {kSecondOfTwo, 512, 256, 0, {2, 16, 16}},
    {kFirstOfTwo, 512, 512, 0, {16, 16, 2}},    {kSecondOfTwo, 512, 512, 1, {16, 16, 2}},
    {kSecondOfTwo, 512, 512, 0, {16, 16, 2}},   {kSingle, 512, 1, 0, {16, 16, 2}},
    {kSingle, 1024, 1, 0, {16, 16, 4}},         {kSingle, 2048, 1, 0, {16, 16, 8}},
    {kSingle, 4096, 1, 0, {16, 16, 16}},        {kFirstOfTwo, 128, 64, 0, {16, 8, 0}},
    {kSecondOfTwo, 64, 128, 0, {16, 4, 0}}};
constexpr int kDirectVariants = (int)(sizeof(kDirectGroups) / sizeof(kDirectGroups[0]));

template <bool FWD>
DirectFn direct_fn(int v) {
  switch (v) {
    case 0: return direct_kernel_f32<FWD, kFirstOfTwo, 128, 128, false, 16, 8, 0>;
    case 1: return direct_kernel_f32<FWD, kSecondOfTwo, 128, 128, false, 16, 8, 0>;
    case 2: return direct_kernel_f32<FWD, kFirstOfTwo, 256, 128, false, 16, 16, 0>;
    case 3: return direct_kernel_f32<FWD, kSecondOfTwo, 128, 256, false, 16, 8, 0>;
    case 4: return direct_kernel_f32<FWD, kFirstOfTwo, 256, 256, false, 16, 16, 0>;
    case 5: return direct_kernel_f32<FWD, kSecondOfTwo, 256, 256, true, 16, 16, 0>;
    case 6: return direct_kernel_f32<FWD, kSecondOfTwo, 256, 256, false, 16, 16, 0>;
    case 7: return direct_kernel_f32<FWD, kFirstOfTwo, 256, 512, false, 16, 16, 0>;
    case 8: return direct_kernel_f32<FWD, kSecondOfTwo, 512, 256, true, 2, 16, 16>;
    case 9: return direct_kernel_f32<FWD, kSecondOfTwo, 512, 256, false, 2, 16, 16>;
    case 10: return direct_kernel_f32<FWD, kFirstOfTwo, 512, 512, false, 16, 16, 2>;
    case 11: return direct_kernel_f32<FWD, kSecondOfTwo, 512, 512, true, 16, 16, 2>;
    case 12: return direct_kernel_f32<FWD, kSecondOfTwo, 512, 512, false, 16, 16, 2>;
    case 13: return direct_kernel_f32<FWD, kSingle, 512, 1, false, 16, 16, 2>;
    case 14: return direct_kernel_f32<FWD, kSingle, 1024, 1, false, 16, 16, 4>;
    case 15: return direct_kernel_f32<FWD, kSingle, 2048, 1, false, 16, 16, 8>;
    case 16: return direct_kernel_f32<FWD, kSingle, 4096, 1, false, 16, 16, 16>;
    case 17: return direct_kernel_f32<FWD, kFirstOfTwo, 128, 64, false, 16, 8, 0>;
    case 18: return direct_kernel_f32<FWD, kSecondOfTwo, 64, 128, false, 16, 4, 0>;
    default: return nullptr;
  }
}

size_t direct_smem(int v) {
  const DirectGroup& d = kDirectGroups[v];
  const int C = direct_width(d.layout, d.M);
  const int tiles = d.r[2] > 0 ? 2 : 1;
  return (size_t)tiles * C * direct_pitch(d.M, C) * sizeof(float2);
}

}  // namespace

int direct_variant_f32(int layout, int M, int nsub, bool comp, const int* radices, int npass) {
  if (npass != 2 && npass != 3) return -1;
  for (int v = 0; v < kDirectVariants; ++v) {
    const DirectGroup& d = kDirectGroups[v];
    if (d.layout != layout || d.M != M || d.nsub != nsub || (d.comp != 0) != comp) continue;
    if ((d.r[2] > 0 ? 3 : 2) != npass) continue;
    bool same = true;
    for (int t = 0; t < npass; ++t) same = same && d.r[t] == radices[t];
    if (same) return v;
  }
  return -1;
}

int direct_cols_variant_f32(int M, const int* radices, int npass) {
  if (npass != 2 && npass != 3) return -1;
  for (int v = 0; v < kDirectColVariants; ++v) {
    const DirectCols& d = kDirectCols[v];
    if (d.M != M || (d.r[2] > 0 ? 3 : 2) != npass) continue;
    bool same = true;
    for (int t = 0; t < npass; ++t) same = same && d.r[t] == radices[t];
    if (same) return v;
  }
  return -1;
}

cudaError_t launch_direct_cols_f32(const GroupDesc& gd, bool fwd, const void* in, void* out,
                                   int variant, cudaStream_t stream) {
  if (variant < 0 || variant >= kDirectColVariants) return cudaErrorInvalidValue;
  const DirectCols& d = kDirectCols[variant];
  GroupDesc g = gd;
  set_divisors(g);
  const int np = d.r[2] > 0 ? 3 : 2;
  bool ok = g.M == d.M && g.npass == np && g.nsub >= 1;
  for (int t = 0; t < np && ok; ++t) ok = g.pass[t].R == d.r[t] && (t == 0) == (g.pass[t].tw == nullptr);
  if (!ok) return cudaErrorInvalidValue;
  const int64_t ntiles = (g.total_sub + 15) / 16;
  if (ntiles == 0) return cudaSuccess;
  if (ntiles > 0x7fffffff) return cudaErrorInvalidValue;
  const DirectFn kern = fwd ? direct_cols_fn<true>(variant) : direct_cols_fn<false>(variant);
  kern<<<(unsigned)ntiles, d.M, direct_cols_smem(variant), stream>>>(
      g, static_cast<const float2*>(in), static_cast<float2*>(out));
  return cudaGetLastError();
}

cudaError_t prepare_direct_kernels_f32() {
  for (int v = 0; v < kDirectColVariants; ++v) {
    const int bytes = (int)direct_cols_smem(v);
    cudaError_t e = cudaFuncSetAttribute(direct_cols_fn<true>(v),
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(direct_cols_fn<false>(v), cudaFuncAttributeMaxDynamicSharedMemorySize,
                             bytes);
    if (e != cudaSuccess) return e;
  }
  for (int v = 0; v < kDirectVariants; ++v) {
    const int bytes = (int)direct_smem(v);
    cudaError_t e = cudaFuncSetAttribute(direct_fn<true>(v),
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(direct_fn<false>(v), cudaFuncAttributeMaxDynamicSharedMemorySize,
                             bytes);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t launch_direct_f32(const GroupDesc& gd, bool fwd, const void* in, void* out,
                              int variant, cudaStream_t stream) {
  if (variant < 0 || variant >= kDirectVariants) return cudaErrorInvalidValue;
  const DirectGroup& d = kDirectGroups[variant];
  GroupDesc g = gd;
  set_divisors(g);
  const int C = direct_width(d.layout, d.M);
  const int np = d.r[2] > 0 ? 3 : 2;
  bool ok = g.M == d.M && g.npass == np;
  for (int t = 0; t < np && ok; ++t) ok = g.pass[t].R == d.r[t];
  // the layout the kernel is compiled for
  if (d.layout == kSingle) {
    ok = ok && g.in_elem == 1 && g.out_elem == 1 && g.in_sub == 0 && g.out_sub == 0 &&
         g.twsub == 0;
  } else {
    ok = ok && g.nsub == d.nsub && g.in_sub == 1 && g.in_elem == d.nsub &&
         (g.twsub != 0) == (d.layout == kSecondOfTwo) &&
         (d.layout == kSecondOfTwo ? (g.out_sub == 1 && g.out_elem == d.nsub)
                                   : (g.out_sub == d.M && g.out_elem == 1)) &&
         g.total_sub % C == 0;
  }
  if (!ok) return cudaErrorInvalidValue;
  const int64_t ntiles = (g.total_sub + C - 1) / C;
  if (ntiles == 0) return cudaSuccess;
  if (ntiles > 0x7fffffff) return cudaErrorInvalidValue;
  const DirectFn kern = fwd ? direct_fn<true>(variant) : direct_fn<false>(variant);
  kern<<<(unsigned)ntiles, direct_threads(d.layout, d.M), direct_smem(variant), stream>>>(
      g, static_cast<const float2*>(in), static_cast<float2*>(out));
  return cudaGetLastError();
}

}  // namespace lfg
