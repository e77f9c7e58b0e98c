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
  if (r2c)
    r2c_kernel<T><<<(unsigned)grid, kGroupThreads, smem, stream>>>(
        d, static_cast<const T*>(in), static_cast<Cx*>(out));
  else
    c2r_kernel<T><<<(unsigned)grid, kGroupThreads, smem, stream>>>(
        d, static_cast<const Cx*>(in), static_cast<T*>(out));
  return cudaGetLastError();
}

}  // namespace

cudaError_t prepare_real_kernels() {
  cudaError_t e;
  if ((e = allow_max_smem(r2c_kernel<double>)) != cudaSuccess) return e;
  if ((e = allow_max_smem(c2r_kernel<double>)) != cudaSuccess) return e;
  if ((e = allow_max_smem(r2c_kernel<float>)) != cudaSuccess) return e;
  return allow_max_smem(c2r_kernel<float>);
}

cudaError_t launch_real(const RealDesc& d, int precision, bool r2c, const void* in, void* out,
                        cudaStream_t stream) {
  return precision == 0 ? launch_real_t<double>(d, r2c, in, out, stream)
                        : launch_real_t<float>(d, r2c, in, out, stream);
}

}  // namespace lfg
