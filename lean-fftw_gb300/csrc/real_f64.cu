// FP64 real-input (r2c) and real-output (c2r) transforms for sm_103a.
//
// lean-fftw runs r2c and c2r in its generic engine as a full complex DFT of the real line and
// of its Hermitian extension (`LineOp.apply`, LeanFFTW/Core/Problem.lean:142-150).  Here a
// real line of even length N = 2M is read as M complex values z[m] = x[2m] + i x[2m+1]
// (one coalesced 16-byte load per pair), transformed with the size-M Stockham passes of the
// fast engine's codelets, and split into the half spectrum in a fused epilogue:
//
//   X[k] = 1/2 (A + B) - i/2 w^k (A - B),  A = Z[k], B = conj Z[M-k], w = exp(-2 pi i / N),
//
// so each line makes one trip through HBM.  c2r runs the same identity backwards in a fused
// prologue, Z'[k] = (H[k] + conj H[M-k]) + i w^-k (H[k] - conj H[M-k]), then the backward
// size-M passes, and stores z as the interleaved real output; the imaginary parts of H[0] and
// H[M] are ignored, as the Hermitian extension of the reference does.  Pairs (k, M-k) share
// their loads and twiddle (w^(M-k) = -conj w^k).  Twiddles come from the exact-integer table
// cos/sin(2 pi k / N), k <= M/2 (halved for r2c).
#include <cuda_runtime.h>

#include "real.h"
#include "stockham_dev.cuh"

namespace lfg {
using namespace dev;
namespace {

__device__ __forceinline__ int64_t real_base(const RealDesc& d, int64_t line) {
  const int64_t b = line / d.rows, r = line - b * d.rows;
  return d.r_off + b * d.r_bdist + r * d.r_rdist;   // doubles
}

__device__ __forceinline__ int64_t cplx_base(const RealDesc& d, int64_t line) {
  const int64_t b = line / d.rows, r = line - b * d.rows;
  return d.c_off + b * d.c_bdist + r * d.c_rdist;   // complex elements
}

__global__ void __launch_bounds__(kGroupThreads)
r2c_kernel_f64(const RealDesc d, const double* in, double2* out) {
  extern __shared__ double2 smem_f64[];
  const GroupDesc& g = d.g;
  const int M = d.M;
  const int64_t l0 = (int64_t)blockIdx.x * g.C;
  const int C = (int)min((int64_t)g.C, d.lines - l0);
  double2* A = smem_f64;
  double2* B = smem_f64 + padded_elems(g.C * M);
  for (int idx = threadIdx.x; idx < C * M; idx += blockDim.x) {
    const int c = idx / M, m = idx - c * M;
    A[spad(idx)] = reinterpret_cast<const double2*>(in + real_base(d, l0 + c))[m];
  }
  __syncthreads();
  const double2* F = run_passes_f64<true>(g, A, B, C, -1);
  // (c/2, s/2) and coefficient 1/2; the adjoint mode uses (c, s) and 1, which doubles the
  // bins 1..M-1 exactly
  const double2* __restrict__ tw = static_cast<const double2*>(d.adjoint ? d.post_full : d.post);
  const double hf = d.adjoint ? 1.0 : 0.5;
  const int half = M / 2;
  for (int idx = threadIdx.x; idx < C * (half + 1); idx += blockDim.x) {
    const int c = idx / (half + 1), k = idx - c * (half + 1);
    const int f0 = c * M;
    double2* o = out + cplx_base(d, l0 + c);
    if (k == 0) {
      const double2 z = F[spad(f0)];
      o[0] = make_double2(__dadd_rn(z.x, z.y), 0.0);
      o[M] = make_double2(__dsub_rn(z.x, z.y), 0.0);
      continue;
    }
    const double2 a = F[spad(f0 + k)], bc = F[spad(f0 + M - k)];
    const double sr = __dadd_rn(a.x, bc.x), si = __dsub_rn(a.y, bc.y);
    const double dr = __dsub_rn(a.x, bc.x), di = __dadd_rn(a.y, bc.y);
    const double2 w = __ldg(tw + k);
    const double P = __fma_rn(w.x, di, -__dmul_rn(w.y, dr));   // (c di - s dr) / 2
    const double Q = __fma_rn(w.y, di, __dmul_rn(w.x, dr));    // (s di + c dr) / 2
    o[k] = make_double2(__fma_rn(hf, sr, P), __fma_rn(hf, si, -Q));
    if (k != M - k) o[M - k] = make_double2(__fma_rn(hf, sr, -P), __fma_rn(-hf, si, -Q));
  }
}

__global__ void __launch_bounds__(kGroupThreads)
c2r_kernel_f64(const RealDesc d, const double2* in, double* out) {
  extern __shared__ double2 smem_f64[];
  const GroupDesc& g = d.g;
  const int M = d.M;
  const int64_t l0 = (int64_t)blockIdx.x * g.C;
  const int C = (int)min((int64_t)g.C, d.lines - l0);
  double2* A = smem_f64;
  double2* B = smem_f64 + padded_elems(g.C * M);
  const double2* __restrict__ tw = static_cast<const double2*>(d.post);   // (c, s)
  const int half = M / 2;
  for (int idx = threadIdx.x; idx < C * (half + 1); idx += blockDim.x) {
    const int c = idx / (half + 1), k = idx - c * (half + 1);
    const double2* h = in + cplx_base(d, l0 + c);
    const int z0 = c * M;
    if (k == 0) {
      const double h0 = h[0].x, hm = h[M].x;   // imaginary parts ignored
      A[spad(z0)] = make_double2(__dadd_rn(h0, hm), __dsub_rn(h0, hm));
      continue;
    }
    double2 a = h[k], bc = h[M - k];
    if (d.adjoint) {   // halve the bins 1..M-1 (exact)
      a = make_double2(__dmul_rn(a.x, 0.5), __dmul_rn(a.y, 0.5));
      bc = make_double2(__dmul_rn(bc.x, 0.5), __dmul_rn(bc.y, 0.5));
    }
    const double sr = __dadd_rn(a.x, bc.x), si = __dsub_rn(a.y, bc.y);
    const double dr = __dsub_rn(a.x, bc.x), di = __dadd_rn(a.y, bc.y);
    const double2 w = __ldg(tw + k);
    const double U = __fma_rn(w.x, di, __dmul_rn(w.y, dr));    // c di + s dr
    const double V = __fma_rn(w.x, dr, -__dmul_rn(w.y, di));   // c dr - s di
    A[spad(z0 + k)] = make_double2(__dsub_rn(sr, U), __dadd_rn(si, V));
    if (k != M - k) A[spad(z0 + M - k)] = make_double2(__dadd_rn(sr, U), __dsub_rn(V, si));
  }
  __syncthreads();
  const double2* F = run_passes_f64<false>(g, A, B, C, -1);
  for (int idx = threadIdx.x; idx < C * M; idx += blockDim.x) {
    const int c = idx / M, m = idx - c * M;
    reinterpret_cast<double2*>(out + real_base(d, l0 + c))[m] = F[spad(idx)];
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

}  // namespace

cudaError_t prepare_real_kernels_f64() {
  cudaError_t e = allow_max_smem(r2c_kernel_f64);
  if (e != cudaSuccess) return e;
  return allow_max_smem(c2r_kernel_f64);
}

cudaError_t launch_real_f64(const RealDesc& rd, bool r2c, const void* in, void* out,
                            cudaStream_t stream) {
  RealDesc d = rd;
  set_divisors(d.g);
  const int64_t grid = (d.lines + d.g.C - 1) / d.g.C;
  if (grid <= 0) return cudaSuccess;
  const size_t smem = 2 * (size_t)padded_elems(d.g.C * d.M) * sizeof(double2);
  if (r2c)
    r2c_kernel_f64<<<(unsigned)grid, kGroupThreads, smem, stream>>>(
        d, static_cast<const double*>(in), static_cast<double2*>(out));
  else
    c2r_kernel_f64<<<(unsigned)grid, kGroupThreads, smem, stream>>>(
        d, static_cast<const double2*>(in), static_cast<double*>(out));
  return cudaGetLastError();
}

}  // namespace lfg
