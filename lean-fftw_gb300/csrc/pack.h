// Gather / scatter between strided (possibly split re/im) layouts and dense row-major complex
// buffers (kernels in pack.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace lfg {

constexpr int kPackMaxDims = 8;

enum PackMode {
  kPackComplex = 0,   // complex values (re at re_off, im at im_off; im_off < 0: imaginary 0)
  kPackReal = 1,      // gather: real values, imaginary part 0; scatter: real parts only
  kPackHerm = 2,      // gather: Hermitian extension of a half spectrum along the last dimension
};

// A tensor of extents n[0..ndims) (row-major on the dense side).  Strided side: element
// (i_0, ..., i_{ndims-1}) at re_off + sum i_k st[k] (and im_off + ...), in real scalars.
// `half`: gather kPackHerm, the strided side's last extent (n/2+1); scatter, when > 0, only
// the first `half` values of the last dimension are written.  `total`: elements moved.
struct PackDesc {
  int ndims;
  int mode;
  int64_t n[kPackMaxDims];
  int64_t st[kPackMaxDims];
  int64_t re_off, im_off;
  int64_t half;
  int64_t total;
};

cudaError_t launch_pack(const PackDesc& d, int precision, const void* src, void* dense,
                        cudaStream_t stream);
cudaError_t launch_unpack(const PackDesc& d, int precision, const void* dense, void* dst,
                          cudaStream_t stream);

}  // namespace lfg
