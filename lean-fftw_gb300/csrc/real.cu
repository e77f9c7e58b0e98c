// Real-input (r2c) and real-output (c2r) transforms for sm_103a, binary64 and binary32.
//
// lean-fftw runs r2c and c2r in its generic engine as a full complex DFT of the real line and
// of its Hermitian extension (`LineOp.apply`, LeanFFTW/Core/Problem.lean:142-150).  Here a
// real line of even length N = 2M is read as M complex values z[m] = x[2m] + i x[2m+1]
// (one coalesced load per pair), transformed with the size-M Stockham passes of the fast
// engine's codelets, and split into the half spectrum in a fused epilogue:
//
//   X[k] = 1/2 (A + B) - i/2 w^k (A - B),  A = Z[k], B = conj Z[M-k], w = exp(-2 pi i / N),
//
// so each line makes one trip through HBM.  c2r runs the same identity backwards in a fused
// prologue, Z'[k] = (H[k] + conj H[M-k]) + i w^-k (H[k] - conj H[M-k]), then the backward
// size-M passes, and stores z as the interleaved real output; the imaginary parts of H[0] and
// H[M] are ignored, as the Hermitian extension of the reference does.  Pairs (k, M-k) share
// their loads and twiddle (w^(M-k) = -conj w^k).  Twiddles come from the exact-integer table
// cos/sin(2 pi k / N), k <= M/2 (halved for r2c); the binary32 variant rounds them once.
#include <cuda_runtime.h>

#include "real.h"

#include "direct_dev.cuh"
#include "stockham_dev.cuh"

namespace lfg {
using namespace dev;
namespace {

__device__ __forceinline__ int64_t real_base(const RealDesc& d, int64_t line) {
  const int64_t b = line / d.rows, r = line - b * d.rows;
  return d.r_off + b * d.r_bdist + r * d.r_rdist;   // real scalars
}

__device__ __forceinline__ int64_t cplx_base(const RealDesc& d, int64_t line) {
  const int64_t b = line / d.rows, r = line - b * d.rows;
  return d.c_off + b * d.c_bdist + r * d.c_rdist;   // complex elements
}

// Additions and multiplications of the split epilogue / prologue; binary64 uses the fused
// forms of the codelets (a*1 + b, a*b + (-0): the same values, at the DFMA issue rate).
template <class T>
struct RealOps;
template <>
struct RealOps<double> {
  double one, nz;
  __device__ __forceinline__ RealOps() { Prec<double>::units(one, nz); }
  __device__ __forceinline__ double add(double a, double b) const { return __fma_rn(a, one, b); }
  __device__ __forceinline__ double sub(double a, double b) const { return __fma_rn(-b, one, a); }
  __device__ __forceinline__ double mul(double a, double b) const { return __fma_rn(a, b, nz); }
};
template <>
struct RealOps<float> {
  __device__ __forceinline__ float add(float a, float b) const { return __fadd_rn(a, b); }
  __device__ __forceinline__ float sub(float a, float b) const { return __fsub_rn(a, b); }
  __device__ __forceinline__ float mul(float a, float b) const { return __fmul_rn(a, b); }
};

template <class T>
__global__ void __launch_bounds__(kGroupThreads)
r2c_kernel(const RealDesc d, const T* in, typename Prec<T>::C* out) {
  using P = Prec<T>;
  using O = RealOps<T>;
  const O ops;
  using Cx = typename P::C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Cx* smem = reinterpret_cast<Cx*>(smem_raw);
  const GroupDesc& g = d.g;
  const int M = d.M;
  const int64_t l0 = (int64_t)blockIdx.x * g.C;
  const int C = (int)min((int64_t)g.C, d.lines - l0);
  const int PM = sub_pitch(M);
  Cx* A = smem;
  Cx* B = smem + tile_elems(g.C, M);
  for (int idx = threadIdx.x; idx < C * M; idx += blockDim.x) {
    const int c = fdiv(idx, g.fd_m), m = idx - c * M;
    A[c * PM + spad(m)] = reinterpret_cast<const Cx*>(in + real_base(d, l0 + c))[m];
  }
  __syncthreads();
  const Cx* F = run_passes<T, true>(g, A, B, C, -1);
  // (c/2, s/2) and coefficient 1/2; the adjoint mode uses (c, s) and 1, which doubles the
  // bins 1..M-1 exactly
  const Cx* __restrict__ tw = static_cast<const Cx*>(d.adjoint ? d.post_full : d.post);
  const T hf = d.adjoint ? T(1) : T(0.5);
  const int half = M / 2;
  for (int idx = threadIdx.x; idx < C * (half + 1); idx += blockDim.x) {
    const int c = idx / (half + 1), k = idx - c * (half + 1);
    const Cx* Fc = F + c * PM;
    Cx* o = out + cplx_base(d, l0 + c);
    if (k == 0) {
      const Cx z = Fc[0];
      o[0] = P::mk(ops.add(z.x, z.y), T(0));
      o[M] = P::mk(ops.sub(z.x, z.y), T(0));
      continue;
    }
    const Cx a = Fc[spad(k)], bc = Fc[spad(M - k)];
    const T sr = ops.add(a.x, bc.x), si = ops.sub(a.y, bc.y);
    const T dr = ops.sub(a.x, bc.x), di = ops.add(a.y, bc.y);
    const Cx w = __ldg(tw + k);
    const T Pp = P::fma(w.x, di, -ops.mul(w.y, dr));   // (c di - s dr) / 2
    const T Q = P::fma(w.y, di, ops.mul(w.x, dr));     // (s di + c dr) / 2
    o[k] = P::mk(P::fma(hf, sr, Pp), P::fma(hf, si, -Q));
    if (k != M - k) o[M - k] = P::mk(P::fma(hf, sr, -Pp), P::fma(-hf, si, -Q));
  }
}

template <class T>
__global__ void __launch_bounds__(kGroupThreads)
c2r_kernel(const RealDesc d, const typename Prec<T>::C* in, T* out) {
  using P = Prec<T>;
  using O = RealOps<T>;
  const O ops;
  using Cx = typename P::C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Cx* smem = reinterpret_cast<Cx*>(smem_raw);
  const GroupDesc& g = d.g;
  const int M = d.M;
  const int64_t l0 = (int64_t)blockIdx.x * g.C;
  const int C = (int)min((int64_t)g.C, d.lines - l0);
  const int PM = sub_pitch(M);
  Cx* A = smem;
  Cx* B = smem + tile_elems(g.C, M);
  const Cx* __restrict__ tw = static_cast<const Cx*>(d.post);   // (c, s)
  const int half = M / 2;
  for (int idx = threadIdx.x; idx < C * (half + 1); idx += blockDim.x) {
    const int c = idx / (half + 1), k = idx - c * (half + 1);
    const Cx* h = in + cplx_base(d, l0 + c);
    Cx* Ac = A + c * PM;
    if (k == 0) {
      const T h0 = h[0].x, hm = h[M].x;   // imaginary parts ignored
      Ac[0] = P::mk(ops.add(h0, hm), ops.sub(h0, hm));
      continue;
    }
    Cx a = h[k], bc = h[M - k];
    if (d.adjoint) {   // halve the bins 1..M-1 (exact)
      a = P::mk(ops.mul(a.x, T(0.5)), ops.mul(a.y, T(0.5)));
      bc = P::mk(ops.mul(bc.x, T(0.5)), ops.mul(bc.y, T(0.5)));
    }
    const T sr = ops.add(a.x, bc.x), si = ops.sub(a.y, bc.y);
    const T dr = ops.sub(a.x, bc.x), di = ops.add(a.y, bc.y);
    const Cx w = __ldg(tw + k);
    const T U = P::fma(w.x, di, ops.mul(w.y, dr));    // c di + s dr
    const T V = P::fma(w.x, dr, -ops.mul(w.y, di));   // c dr - s di
    Ac[spad(k)] = P::mk(ops.sub(sr, U), ops.add(si, V));
    if (k != M - k) Ac[spad(M - k)] = P::mk(ops.add(sr, U), ops.sub(V, si));
  }
  __syncthreads();
  const Cx* F = run_passes<T, false>(g, A, B, C, -1);
  for (int idx = threadIdx.x; idx < C * M; idx += blockDim.x) {
    const int c = fdiv(idx, g.fd_m), m = idx - c * M;
    reinterpret_cast<Cx*>(out + real_base(d, l0 + c))[m] = F[c * PM + spad(m)];
  }
}

// The rows of a binary32 r2c plan with a register-staged variant (M = N / 2 complex points a
// power of two): C = 4096 / M rows per CTA of 256 threads; the first pass loads its
// butterflies' inputs straight from the rows, the later passes run through shared tiles, and
// the split epilogue reads the last tile and stores the half spectrum -- the operations of
// r2c_kernel above on the same operands, so the same bits.
template <int M, int R0, int R1, int R2>
__global__ void __launch_bounds__(256, 3)
r2c_rows_direct_f32(const RealDesc d, const float* in, float2* out) {
  using namespace dfx;
  using P = Prec<float>;
  const RealOps<float> ops;
  constexpr int C = kDirectPoints / M, T = 256, PM = sub_pitch(M), MR0 = M / R0;
  static_assert(M == R0 * R1 * (R2 > 0 ? R2 : 1) && C * MR0 == T, "one first-pass butterfly per thread");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* A = reinterpret_cast<float2*>(smem_raw);
  float2* B = A + C * PM;
  const GroupDesc& g = d.g;
  const int64_t l0 = (int64_t)blockIdx.x * C;
  const int count = (int)min((int64_t)C, d.lines - l0);
  const int c0 = (int)threadIdx.x / MR0;   // the thread's row in the first pass
  const bool valid = c0 < count;
  const float2* tin = valid ? reinterpret_cast<const float2*>(in + real_base(d, l0 + c0)) : nullptr;
  direct_pass<true, M, C, PM, T, R0, 1, 0, false, 0, kFromRowsRT, kToTile>(
      nullptr, 0, nullptr, A, nullptr, 0, nullptr, 0, count, true, 1.0f, tin, nullptr, 0, valid);
  __syncthreads();
  direct_pass<true, M, C, PM, T, R1, R0, 0, false, 1, kFromTile, kToTile>(
      nullptr, 0, A, B, nullptr, 0, static_cast<const float2*>(g.pass[1].tw), 0, count, true, 1.0f);
  __syncthreads();
  const float2* F = B;
  if constexpr (R2 > 0) {
    direct_pass<true, M, C, PM, T, R2, R0 * R1, 0, false, 1, kFromTile, kToTile>(
        nullptr, 0, B, A, nullptr, 0, static_cast<const float2*>(g.pass[2].tw), 0, count, true,
        1.0f);
    __syncthreads();
    F = A;
  }
  const float2* __restrict__ tw = static_cast<const float2*>(d.adjoint ? d.post_full : d.post);
  const float hf = d.adjoint ? 1.0f : 0.5f;
  constexpr int half = M / 2;
  for (int idx = threadIdx.x; idx < count * (half + 1); idx += T) {
    const int c = idx / (half + 1), k = idx - c * (half + 1);
    const float2* Fc = F + c * PM;
    float2* o = out + cplx_base(d, l0 + c);
    if (k == 0) {
      const float2 z = Fc[0];
      o[0] = P::mk(ops.add(z.x, z.y), 0.0f);
      o[M] = P::mk(ops.sub(z.x, z.y), 0.0f);
      continue;
    }
    const float2 a = Fc[spad(k)], bc = Fc[spad(M - k)];
    const float sr = ops.add(a.x, bc.x), si = ops.sub(a.y, bc.y);
    const float dr = ops.sub(a.x, bc.x), di = ops.add(a.y, bc.y);
    const float2 w = __ldg(tw + k);
    const float Pp = P::fma(w.x, di, -ops.mul(w.y, dr));
    const float Q = P::fma(w.y, di, ops.mul(w.x, dr));
    o[k] = P::mk(P::fma(hf, sr, Pp), P::fma(hf, si, -Q));
    if (k != M - k) o[M - k] = P::mk(P::fma(hf, sr, -Pp), P::fma(-hf, si, -Q));
  }
}

using RowsFn = void (*)(const RealDesc, const float*, float2*);
struct RowsVariant {
  int M, r[3];
};
constexpr RowsVariant kRowsVariants[] = {
    {128, {16, 8, 0}}, {256, {16, 16, 0}}, {512, {16, 16, 2}}, {1024, {16, 16, 4}}};
constexpr int kNRowsVariants = (int)(sizeof(kRowsVariants) / sizeof(kRowsVariants[0]));

RowsFn rows_fn(int v) {
  switch (v) {
    case 0: return r2c_rows_direct_f32<128, 16, 8, 0>;
    case 1: return r2c_rows_direct_f32<256, 16, 16, 0>;
    case 2: return r2c_rows_direct_f32<512, 16, 16, 2>;
    case 3: return r2c_rows_direct_f32<1024, 16, 16, 4>;
    default: return nullptr;
  }
}

size_t rows_smem(int v) {
  const int M = kRowsVariants[v].M;
  return 2 * (size_t)(dfx::kDirectPoints / M) * sub_pitch(M) * sizeof(float2);
}

template <class K>
cudaError_t allow_max_smem(K kern) {
  cudaFuncAttributes a;
  cudaError_t e = cudaFuncGetAttributes(&a, kern);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)(kMaxSmemBytes - a.sharedSizeBytes));
}

template <class T>
cudaError_t launch_real_t(const RealDesc& rd, bool r2c, const void* in, void* out,
                          cudaStream_t stream) {
  using Cx = typename Prec<T>::C;
  RealDesc d = rd;
  set_divisors(d.g);
  const int64_t grid = (d.lines + d.g.C - 1) / d.g.C;
  if (grid <= 0) return cudaSuccess;
  const size_t smem = 2 * (size_t)tile_elems(d.g.C, d.M) * sizeof(Cx);
  if (r2c && sizeof(T) == 4 && d.direct >= 0 && d.direct < kNRowsVariants) {
    const int C = dfx::kDirectPoints / kRowsVariants[d.direct].M;
    const int64_t tiles = (d.lines + C - 1) / C;
    rows_fn(d.direct)<<<(unsigned)tiles, 256, rows_smem(d.direct), stream>>>(
        d, reinterpret_cast<const float*>(in), reinterpret_cast<float2*>(out));
  } else if (r2c)
    r2c_kernel<T><<<(unsigned)grid, kGroupThreads, smem, stream>>>(
        d, static_cast<const T*>(in), static_cast<Cx*>(out));
  else
    c2r_kernel<T><<<(unsigned)grid, kGroupThreads, smem, stream>>>(
        d, static_cast<const Cx*>(in), static_cast<T*>(out));
  return cudaGetLastError();
}

}  // namespace

int r2c_rows_variant_f32(int M, const int* radices, int npass) {
  for (int v = 0; v < kNRowsVariants; ++v) {
    const RowsVariant& rv = kRowsVariants[v];
    if (rv.M != M || (rv.r[2] > 0 ? 3 : 2) != npass) continue;
    bool same = true;
    for (int t = 0; t < npass; ++t) same = same && rv.r[t] == radices[t];
    if (same) return v;
  }
  return -1;
}

cudaError_t prepare_real_kernels() {
  cudaError_t e;
  if ((e = allow_max_smem(r2c_kernel<double>)) != cudaSuccess) return e;
  if ((e = allow_max_smem(c2r_kernel<double>)) != cudaSuccess) return e;
  if ((e = allow_max_smem(r2c_kernel<float>)) != cudaSuccess) return e;
  for (int v = 0; v < kNRowsVariants; ++v)
    if ((e = cudaFuncSetAttribute(rows_fn(v), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)rows_smem(v))) != cudaSuccess)
      return e;
  return allow_max_smem(c2r_kernel<float>);
}

cudaError_t launch_real(const RealDesc& d, int precision, bool r2c, const void* in, void* out,
                        cudaStream_t stream) {
  return precision == 0 ? launch_real_t<double>(d, r2c, in, out, stream)
                        : launch_real_t<float>(d, r2c, in, out, stream);
}

}  // namespace lfg
