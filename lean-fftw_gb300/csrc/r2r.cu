// Real-to-real transforms (lean-fftw's eleven r2r kinds), binary64 and binary32.
//
// lean-fftw computes an r2r line as an exact symmetric embedding of the real input into a
// complex sequence of length M = embedSize(kind, n), a complex DFT of that length (backward
// for hc2r, whose halfcomplex input is first expanded to its Hermitian extension), and an
// exact extraction of the outputs (`R2RKind.embed` / `extract` and `LineOp.apply`,
// LeanFFTW/Core/Problem.lean:64-112, 151-163).  Here the embedding and the extraction are two
// element-wise kernels around the library's own complex transform; they move data only
// (copies and sign flips), so the arithmetic is that of the complex transform.
#include <cuda_runtime.h>

#include <algorithm>

#include "r2r.h"
#include "stockham_dev.cuh"

namespace lfg {
using namespace dev;
namespace {

// Start of line l = l1 + nl1 * l2 (l1 < nl1) on one side, in real scalars.
__device__ __forceinline__ int64_t line_base(int line, const R2RDesc& d, bool out) {
  const int q = d.nl1 >= d.lines ? 0 : fdiv(line, d.fd_nl1);
  const int64_t l1 = line - (int64_t)q * d.nl1;
  return out ? d.out_off + l1 * d.out_dist + q * d.out_dist2
             : d.in_off + l1 * d.in_dist + q * d.in_dist2;
}

// z[line*M + i] = the embedding of input line `line` at i (complex, imaginary part 0 except
// for hc2r, whose Hermitian extension is complex).
template <class T>
__global__ void r2r_embed(const R2RDesc d, const T* __restrict__ in, typename Prec<T>::C* z) {
  using Cx = typename Prec<T>::C;
  const int total = (int)(d.lines * d.M);    // < 2^31 (planner)
  const int64_t n = d.n, M = d.M;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += gridDim.x * blockDim.x) {
    const int line = fdiv(idx, d.fd_m);
    const int64_t i = idx - (int64_t)line * M;
    const T* x = in + line_base(line, d, false);
    const int64_t s = d.in_stride;
    auto X = [&](int64_t j) { return x[j * s]; };
    T re = T(0), im = T(0);
    switch (d.kind) {
      case kR2HC:
      case kDHT:
        re = X(i);
        break;
      case kHC2R: {
        // halfcomplex: r_k at k (k <= n/2), i_k at n-k (0 < k < n-k); Hermitian extension
        const int64_t k = i <= n / 2 ? i : n - i;
        re = X(k);
        const T ik = (0 < k && k < n - k) ? X(n - k) : T(0);
        im = i <= n / 2 ? ik : -ik;
        break;
      }
      case kREDFT00:
        re = i < n ? X(i) : X(M - i);
        break;
      case kRODFT00:
        if (1 <= i && i <= n) re = X(i - 1);
        else if (n + 2 <= i) re = -X(M - i - 1);
        break;
      case kREDFT10:
        if (i & 1) re = i < 2 * n ? X(i / 2) : X((M - i) / 2);
        break;
      case kRODFT10:
        if (i & 1) re = i < 2 * n ? X(i / 2) : -X((M - i) / 2);
        break;
      case kREDFT11:
        if (i & 1) {
          if (i < 2 * n) re = X(i / 2);
          else if (6 * n < i) re = X((M - i) / 2);
        }
        break;
      case kRODFT11:
        if (i & 1) {
          if (i < 2 * n) re = X(i / 2);
          else if (6 * n < i) re = -X((M - i) / 2);
        }
        break;
      case kREDFT01:
        if (i < n) re = X(i);
        else if (3 * n < i) re = X(M - i);
        break;
      case kRODFT01:
        if (1 <= i && i <= n) re = X(i - 1);
        else if (3 * n < i) re = -X(M - i - 1);
        break;
      default:
        break;
    }
    z[idx] = Prec<T>::mk(re, im);
  }
}

// out line `line`, element j: the extraction from F (line*M .. line*M + M-1).
template <class T>
__global__ void r2r_extract(const R2RDesc d, const typename Prec<T>::C* __restrict__ F, T* out) {
  const int total = (int)(d.lines * d.n);
  const int64_t n = d.n, M = d.M;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += gridDim.x * blockDim.x) {
    const int line = fdiv(idx, d.fd_n);
    const int64_t j = idx - (int64_t)line * n;
    const auto* f = F + (int64_t)line * M;
    T v;
    switch (d.kind) {
      case kR2HC:
        v = j <= n / 2 ? f[j].x : f[n - j].y;
        break;
      case kHC2R:
      case kREDFT00:
      case kREDFT10:
        v = f[j].x;
        break;
      case kDHT:
        v = f[j].x - f[j].y;
        break;
      case kREDFT01:
      case kREDFT11:
        v = f[2 * j + 1].x;
        break;
      case kRODFT00:
      case kRODFT10:
        v = -f[j + 1].y;
        break;
      default:   // kRODFT01, kRODFT11
        v = -f[2 * j + 1].y;
        break;
    }
    out[line_base(line, d, true) + j * d.out_stride] = v;
  }
}

unsigned grid_for(int64_t total) {
  const int64_t b = (total + 255) / 256;
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(b, 152 * 16));
}

}  // namespace

cudaError_t launch_r2r_embed(const R2RDesc& d, int precision, const void* in, void* z,
                             cudaStream_t stream) {
  const unsigned grid = grid_for(d.lines * d.M);
  if (precision == 0)
    r2r_embed<double><<<grid, 256, 0, stream>>>(d, static_cast<const double*>(in),
                                                 static_cast<double2*>(z));
  else
    r2r_embed<float><<<grid, 256, 0, stream>>>(d, static_cast<const float*>(in),
                                                static_cast<float2*>(z));
  return cudaGetLastError();
}

cudaError_t launch_r2r_extract(const R2RDesc& d, int precision, const void* F, void* out,
                               cudaStream_t stream) {
  const unsigned grid = grid_for(d.lines * d.n);
  if (precision == 0)
    r2r_extract<double><<<grid, 256, 0, stream>>>(d, static_cast<const double2*>(F),
                                                   static_cast<double*>(out));
  else
    r2r_extract<float><<<grid, 256, 0, stream>>>(d, static_cast<const float2*>(F),
                                                  static_cast<float*>(out));
  return cudaGetLastError();
}

}  // namespace lfg
