// Bluestein (chirp-z) transforms for sizes with a prime factor above 13: descriptor and
// launchers of the element-wise kernels (chirp.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "stockham.h"

namespace lfg {

// Lines l = l1 + nl1 * l2 (l1 < nl1) of n complex elements: input at in_off + l1*in_dist +
// l2*in_dist2, element stride in_stride (complex elements), likewise for the output.  The
// convolution buffer holds L complex elements per line, back to back.
struct ChirpDesc {
  int64_t n, L, lines, nl1;
  int64_t in_off, in_stride, in_dist, in_dist2;
  int64_t out_off, out_stride, out_dist, out_dist2;
  FastDiv fd_L, fd_n, fd_nl1;
  const void* chirp;    // c_m = exp(s pi i m^2 / n), m < n
  const void* bhat;     // forward transform (length L) of conj(c) placed circularly
};

cudaError_t launch_chirp_pre(const ChirpDesc& d, int precision, const void* in, void* buf,
                             cudaStream_t stream);
cudaError_t launch_chirp_mul(const ChirpDesc& d, int precision, void* buf, cudaStream_t stream);
cudaError_t launch_chirp_post(const ChirpDesc& d, int precision, const void* buf, void* out,
                              cudaStream_t stream);

}  // namespace lfg
