// Complex transforms of sizes with a prime factor above 13 (Bluestein's chirp-z algorithm),
// binary64 and binary32.
//
// lean-fftw's fast engine only plans 13-smooth sizes; its generic engine takes any n, with a
// direct O(p^2) sum for each prime factor p (Core/Alg.lean:31-105).  On the GPU such sizes
// go through Bluestein's identity jk = (j^2 + k^2 - (k-j)^2) / 2:
//
//   X_k = c_k * sum_j (x_j c_j) conj(c_{k-j}),   c_m = exp(s pi i m^2 / n),
//
// a circular convolution of length L >= 2n-1 (13-smooth), computed with the library's own
// transforms: a forward transform of the chirped, zero-padded input, a pointwise product with
// the precomputed transform of conj(c), and a backward transform scaled by 1/L in its store.
// The chirp c_m comes from the exact-integer table of cos/sin(2 pi t / 2n), t = m^2 mod 2n, so
// it is correctly rounded.  The three element-wise steps are the kernels below.
#include <cuda_runtime.h>

#include <algorithm>

#include "chirp.h"
#include "stockham_dev.cuh"

namespace lfg {
using namespace dev;
namespace {

__device__ __forceinline__ int64_t chirp_line_base(int line, const ChirpDesc& d, bool out) {
  const int q = d.nl1 >= d.lines ? 0 : fdiv(line, d.fd_nl1);
  const int64_t l1 = line - (int64_t)q * d.nl1;
  return out ? d.out_off + l1 * d.out_dist + q * d.out_dist2
             : d.in_off + l1 * d.in_dist + q * d.in_dist2;
}

template <class T>
__device__ __forceinline__ typename Prec<T>::C cmul(typename Prec<T>::C a, typename Prec<T>::C b) {
  using P = Prec<T>;
  return P::mk(P::fma(a.x, b.x, -P::mul(a.y, b.y)), P::fma(a.x, b.y, P::mul(a.y, b.x)));
}

// buf[line*L + j] = x_j c_j for j < n, 0 for n <= j < L
template <class T>
__global__ void chirp_pre(const ChirpDesc d, const typename Prec<T>::C* __restrict__ in,
                          typename Prec<T>::C* __restrict__ buf) {
  using Cx = typename Prec<T>::C;
  const Cx* __restrict__ c = static_cast<const Cx*>(d.chirp);
  const int total = (int)(d.lines * d.L);
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += gridDim.x * blockDim.x) {
    const int line = fdiv(idx, d.fd_L);
    const int j = idx - line * (int)d.L;
    Cx v = Prec<T>::mk(T(0), T(0));
    if (j < d.n) v = cmul<T>(in[chirp_line_base(line, d, false) + (int64_t)j * d.in_stride], __ldg(c + j));
    buf[idx] = v;
  }
}

// buf[line*L + j] *= bhat[j]
template <class T>
__global__ void chirp_mul(const ChirpDesc d, typename Prec<T>::C* __restrict__ buf) {
  using Cx = typename Prec<T>::C;
  const Cx* __restrict__ bh = static_cast<const Cx*>(d.bhat);
  const int total = (int)(d.lines * d.L);
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += gridDim.x * blockDim.x) {
    const int line = fdiv(idx, d.fd_L);
    const int j = idx - line * (int)d.L;
    buf[idx] = cmul<T>(buf[idx], __ldg(bh + j));
  }
}

// out_k = c_k conv_k for k < n
template <class T>
__global__ void chirp_post(const ChirpDesc d, const typename Prec<T>::C* __restrict__ buf,
                           typename Prec<T>::C* __restrict__ out) {
  using Cx = typename Prec<T>::C;
  const Cx* __restrict__ c = static_cast<const Cx*>(d.chirp);
  const int total = (int)(d.lines * d.n);
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += gridDim.x * blockDim.x) {
    const int line = fdiv(idx, d.fd_n);
    const int k = idx - line * (int)d.n;
    out[chirp_line_base(line, d, true) + (int64_t)k * d.out_stride] =
        cmul<T>(__ldg(c + k), buf[(int64_t)line * d.L + k]);
  }
}

unsigned grid_for(int64_t total) {
  const int64_t b = (total + 255) / 256;
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(b, 152 * 16));
}

}  // namespace

cudaError_t launch_chirp_pre(const ChirpDesc& d, int precision, const void* in, void* buf,
                             cudaStream_t stream) {
  const unsigned g = grid_for(d.lines * d.L);
  if (precision == 0)
    chirp_pre<double><<<g, 256, 0, stream>>>(d, static_cast<const double2*>(in), static_cast<double2*>(buf));
  else
    chirp_pre<float><<<g, 256, 0, stream>>>(d, static_cast<const float2*>(in), static_cast<float2*>(buf));
  return cudaGetLastError();
}

cudaError_t launch_chirp_mul(const ChirpDesc& d, int precision, void* buf, cudaStream_t stream) {
  const unsigned g = grid_for(d.lines * d.L);
  if (precision == 0) chirp_mul<double><<<g, 256, 0, stream>>>(d, static_cast<double2*>(buf));
  else chirp_mul<float><<<g, 256, 0, stream>>>(d, static_cast<float2*>(buf));
  return cudaGetLastError();
}

cudaError_t launch_chirp_post(const ChirpDesc& d, int precision, const void* buf, void* out,
                              cudaStream_t stream) {
  const unsigned g = grid_for(d.lines * d.n);
  if (precision == 0)
    chirp_post<double><<<g, 256, 0, stream>>>(d, static_cast<const double2*>(buf), static_cast<double2*>(out));
  else
    chirp_post<float><<<g, 256, 0, stream>>>(d, static_cast<const float2*>(buf), static_cast<float2*>(out));
  return cudaGetLastError();
}

}  // namespace lfg
