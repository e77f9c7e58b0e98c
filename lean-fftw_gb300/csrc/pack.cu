// Gather / scatter between arbitrary strided layouts and dense row-major complex buffers,
// binary64 and binary32.
//
// lean-fftw's problem description allows any strides and split real/imaginary arrays
// (separate bases, `inRe`/`inIm`, LeanFFTW/FFI.lean:13-21, Core/Problem.lean:170-282).  The
// kernels work on interleaved data; a problem they do not take directly is gathered into a
// dense row-major complex buffer, transformed there, and scattered back.  On GB300 the binary64
// transforms are bound by the FP64 pipe, not by HBM, so the two extra passes over memory cost
// little.  The gather can also build the complex input of a real transform (imaginary part 0)
// or the Hermitian extension of a half spectrum along the last dimension, and the scatter can
// keep only the first n/2+1 values of the last dimension or only the real parts: together they
// run any rdft2 problem through complex transforms, as the reference's generic engine does
// (`LineOp.apply`, Core/Problem.lean:142-150).
#include <cuda_runtime.h>

#include <algorithm>

#include "pack.h"
#include "stockham_dev.cuh"

namespace lfg {
using namespace dev;
namespace {

// Offset (real scalars) of the element at dense index q on the strided side, for extents ext.
__device__ __forceinline__ int64_t strided_offset(int64_t q, const PackDesc& d, const int64_t* ext) {
  int64_t off = 0;
  for (int k = d.ndims - 1; k >= 0; --k) {
    const int64_t i = q % ext[k];
    q /= ext[k];
    off += i * d.st[k];
  }
  return off;
}

template <class T>
__global__ void pack_kernel(const PackDesc d, const T* __restrict__ src, typename Prec<T>::C* dst) {
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < d.total;
       q += (int64_t)gridDim.x * blockDim.x) {
    T re, im;
    if (d.mode == kPackHerm) {
      // Hermitian extension along the last dimension (lean-fftw `hermExt`,
      // Core/Problem.lean:137-138): k <= n/2 read directly, else conj of element n - k of the
      // same row; the source has extents n[0..last-1] x half
      const int last = d.ndims - 1;
      const int64_t k = q % d.n[last];
      int64_t row = q / d.n[last];
      const bool mirror = k >= d.half;
      int64_t off = (mirror ? d.n[last] - k : k) * d.st[last];
      for (int j = last - 1; j >= 0; --j) {
        off += (row % d.n[j]) * d.st[j];
        row /= d.n[j];
      }
      re = src[d.re_off + off];
      im = d.im_off >= 0 ? src[d.im_off + off] : T(0);
      if (mirror) im = -im;
    } else {
      const int64_t off = strided_offset(q, d, d.n);
      re = src[d.re_off + off];
      im = (d.mode == kPackReal || d.im_off < 0) ? T(0) : src[d.im_off + off];
    }
    dst[q] = Prec<T>::mk(re, im);
  }
}

template <class T>
__global__ void unpack_kernel(const PackDesc d, const typename Prec<T>::C* __restrict__ src, T* dst) {
  // iterate over the strided (output) side's extents: n, with the last one `half` when set
  int64_t ext[kPackMaxDims];
  for (int k = 0; k < d.ndims; ++k) ext[k] = d.n[k];
  if (d.half > 0) ext[d.ndims - 1] = d.half;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < d.total;
       q += (int64_t)gridDim.x * blockDim.x) {
    int64_t off = 0, dq = 0, mul = 1, t = q;
    for (int k = d.ndims - 1; k >= 0; --k) {
      const int64_t i = t % ext[k];
      t /= ext[k];
      off += i * d.st[k];
      dq += i * mul;
      mul *= d.n[k];
    }
    const auto v = src[dq];
    dst[d.re_off + off] = v.x;
    if (d.mode != kPackReal && d.im_off >= 0) dst[d.im_off + off] = v.y;
  }
}

unsigned grid_for(int64_t total) {
  const int64_t b = (total + 255) / 256;
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(b, 152 * 16));
}

}  // namespace

cudaError_t launch_pack(const PackDesc& d, int precision, const void* src, void* dense,
                        cudaStream_t stream) {
  const unsigned g = grid_for(d.total);
  if (precision == 0)
    pack_kernel<double><<<g, 256, 0, stream>>>(d, static_cast<const double*>(src), static_cast<double2*>(dense));
  else
    pack_kernel<float><<<g, 256, 0, stream>>>(d, static_cast<const float*>(src), static_cast<float2*>(dense));
  return cudaGetLastError();
}

cudaError_t launch_unpack(const PackDesc& d, int precision, const void* dense, void* dst,
                          cudaStream_t stream) {
  const unsigned g = grid_for(d.total);
  if (precision == 0)
    unpack_kernel<double><<<g, 256, 0, stream>>>(d, static_cast<const double2*>(dense), static_cast<double*>(dst));
  else
    unpack_kernel<float><<<g, 256, 0, stream>>>(d, static_cast<const float2*>(dense), static_cast<float*>(dst));
  return cudaGetLastError();
}

}  // namespace lfg
