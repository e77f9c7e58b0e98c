// Real-input / real-output transforms (kernels in real.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "stockham.h"

namespace lfg {

// Lines of a real transform of even size N = 2M: line L = b * rows + r (b: vector index, r:
// row of a rank-2 transform, rows = 1 for rank 1).  The real side of line L starts at double
// r_off + b*r_bdist + r*r_rdist (even, so pairs load as one complex value) with unit stride;
// the complex side (M+1 values) at complex element c_off + b*c_bdist + r*c_rdist.
struct RealDesc {
  GroupDesc g;                 // the size-M passes, one group (nsub = 1, tile of g.C lines)
  int64_t lines;
  int64_t rows;
  int64_t r_off, r_bdist, r_rdist;
  int64_t c_off, c_bdist, c_rdist;
  const void* post;            // (cos, sin)(2 pi k / N), k = 0..M/2 (r2c: both halved)
  const void* post_full;       // (cos, sin)(2 pi k / N) unhalved (r2c adjoint mode)
  int M;
  // Adjoint scaling of the cotangent, exact (powers of two): r2c doubles the bins 1..M-1 of
  // its output (the gradient of c2r); c2r halves the bins 1..M-1 of its input (the gradient
  // of r2c).  0 = plain transform.
  int adjoint;
  // binary32 r2c rows: the register-staged kernel of r2c_rows_variant_f32 (-1: r2c_kernel)
  int direct = -1;
};

cudaError_t prepare_real_kernels();
// The register-staged binary32 r2c row kernel for M = N / 2 points with these radices
// (128: 16.8, 256: 16.16, 512: 16.16.2, 1024: 16.16.4), or -1.
int r2c_rows_variant_f32(int M, const int* radices, int npass);
// precision 0: binary64 (double lines, double2 spectrum); 1: binary32 (float, float2)
cudaError_t launch_real(const RealDesc& d, int precision, bool r2c, const void* in, void* out,
                        cudaStream_t stream);

}  // namespace lfg
