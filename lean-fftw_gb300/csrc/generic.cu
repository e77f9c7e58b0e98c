// The generic engine's mixed-radix transform, for sizes with a prime factor above 13 (binary64
// bit for bit; binary32 the same steps in binary32).
//
// lean-fftw's generic engine computes `exec floatOps (mkPlan floatOps fwd (primeFactors n))`
// (LeanFFTW/Core/Alg.lean:236-254): decimation in time over the prime factors f_0 <= f_1 <=
// ..., each level a direct sum over its factor, twiddles cosSin2Pi from the exact table with
// the imaginary part negated (never to -0) for the forward direction, and the textbook
// complex product with four rounded products (Core/FloatOps.lean:52-58).  Unrolling the
// recursion: with n_i = f_i ... f_last and P_i = n / n_i, level i holds P_i sub-problems
// Y_i[t][k] (t < P_i, k < n_i), and
//
//   Y_i[t][k] = sum_{j < f_i} w(j k mod n_i, n_i) * Y_{i+1}[t + P_i j][k mod n_{i+1}],
//
// summed from zero in the order j = 0, 1, ..., with Y_last+1[t][0] = x[t] and X = Y_0[0].
// One CTA runs every level of one line in shared memory (n <= 4096), so each output element
// goes through exactly the reference's operations.
#include <cuda_runtime.h>

#include "generic.h"
#include "stockham_dev.cuh"

namespace lfg {
using namespace dev;
namespace {

template <class T, bool FWD>
__global__ void __launch_bounds__(256) generic_kernel(const GenericDesc d, const typename Prec<T>::C* in,
                                                     typename Prec<T>::C* out) {
  using P = Prec<T>;
  using Cx = typename P::C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Cx* A = reinterpret_cast<Cx*>(smem_raw);
  Cx* B = A + d.n;
  const Cx* __restrict__ tab = static_cast<const Cx*>(d.tab);
  const int n = d.n;
  const int64_t line = blockIdx.x;
  const int q = d.nl1 >= d.lines ? 0 : (int)(line / d.nl1);
  const int64_t l1 = line - (int64_t)q * d.nl1;
  const Cx* x = in + l1 * d.in_dist + q * d.in_dist2;
  Cx* y = out + l1 * d.out_dist + q * d.out_dist2;
  for (int t = threadIdx.x; t < n; t += blockDim.x) A[t] = x[(int64_t)t * d.in_stride];
  __syncthreads();
  // Y_{i+1} in A (layout [t][k], t < P_{i+1}, k < n_{i+1}), Y_i into B
  for (int i = d.nf - 1; i >= 0; --i) {
    const int f = d.f[i];
    const int ni = d.ni[i], ni1 = ni / f;    // n_i and n_{i+1}
    const int Pi = n / ni;
    for (int idx = threadIdx.x; idx < n; idx += blockDim.x) {
      const int t = idx / ni, k = idx - t * ni;
      const int kk = k % ni1;
      T accr = T(0), acci = T(0);
      for (int j = 0; j < f; ++j) {
        const int e = (int)(((int64_t)j * k) % ni);
        const Cx w = __ldg(tab + (int64_t)e * Pi);
        const T wr = w.x;
        const T wi = FWD ? (w.y == T(0) ? T(0) : -w.y) : w.y;
        const Cx v = A[(t + Pi * j) * ni1 + kk];
        const T p1 = P::mul(wr, v.x), p2 = P::mul(wi, v.y), p3 = P::mul(wr, v.y), p4 = P::mul(wi, v.x);
        accr = P::add(accr, P::sub(p1, p2));
        acci = P::add(acci, P::add(p3, p4));
      }
      B[idx] = P::mk(accr, acci);
    }
    __syncthreads();
    Cx* tmp = A;
    A = B;
    B = tmp;
  }
  const bool unit = d.scale == 1.0;
  const T sc = (T)d.scale;
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    const Cx v = A[k];
    y[(int64_t)k * d.out_stride] = unit ? v : P::mk(P::mul(v.x, sc), P::mul(v.y, sc));
  }
}

template <class K>
cudaError_t allow_smem(K kern) {
  cudaFuncAttributes a;
  cudaError_t e = cudaFuncGetAttributes(&a, kern);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)(kMaxSmemBytes - a.sharedSizeBytes));
}

}  // namespace

cudaError_t prepare_generic_kernels() {
  cudaError_t e;
  if ((e = allow_smem(generic_kernel<double, true>)) != cudaSuccess) return e;
  if ((e = allow_smem(generic_kernel<double, false>)) != cudaSuccess) return e;
  if ((e = allow_smem(generic_kernel<float, true>)) != cudaSuccess) return e;
  return allow_smem(generic_kernel<float, false>);
}

cudaError_t launch_generic(const GenericDesc& d, int precision, bool fwd, const void* in, void* out,
                           cudaStream_t stream) {
  if (d.lines <= 0) return cudaSuccess;
  const unsigned grid = (unsigned)d.lines;
  if (precision == 0) {
    const size_t smem = 2 * (size_t)d.n * sizeof(double2);
    auto k = fwd ? generic_kernel<double, true> : generic_kernel<double, false>;
    k<<<grid, 256, smem, stream>>>(d, static_cast<const double2*>(in), static_cast<double2*>(out));
  } else {
    const size_t smem = 2 * (size_t)d.n * sizeof(float2);
    auto k = fwd ? generic_kernel<float, true> : generic_kernel<float, false>;
    k<<<grid, 256, smem, stream>>>(d, static_cast<const float2*>(in), static_cast<float2*>(out));
  }
  return cudaGetLastError();
}

}  // namespace lfg
