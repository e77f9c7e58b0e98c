// Real-to-real transforms: descriptors and launchers of the embedding / extraction kernels
// (kernels in r2r.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "stockham.h"

namespace lfg {

// libbench2's r2r kind numbering, as in lean-fftw's FFI encoding (LeanFFTW/FFI.lean:29-31).
enum R2RKindCode {
  kR2HC = 0, kHC2R = 1, kDHT = 2,
  kREDFT00 = 3, kREDFT01 = 4, kREDFT10 = 5, kREDFT11 = 6,
  kRODFT00 = 7, kRODFT01 = 8, kRODFT10 = 9, kRODFT11 = 10,
};

// Size of the complex DFT of the embedding (lean-fftw `R2RKind.embedSize`,
// LeanFFTW/Core/Problem.lean:66-72); 0 for an invalid kind or size.
inline int64_t r2r_embed_size(int kind, int64_t n) {
  switch (kind) {
    case kR2HC: case kHC2R: case kDHT: return n;
    case kREDFT00: return n >= 2 ? 2 * (n - 1) : 0;
    case kRODFT00: return 2 * (n + 1);
    case kREDFT10: case kREDFT01: case kRODFT10: case kRODFT01: return 4 * n;
    case kREDFT11: case kRODFT11: return 8 * n;
    default: return 0;
  }
}

// One batch of r2r lines: line l = l1 + nl1 * l2 (l1 < nl1) starts at off + l1*dist +
// l2*dist2 on each side and has n elements `stride` apart (real scalars).  The embedding of
// line l occupies z[l*M .. l*M + M-1] of a dense complex buffer.
struct R2RDesc {
  int kind;
  int64_t n, M, lines, nl1;
  int64_t in_off, in_stride, in_dist, in_dist2;
  int64_t out_off, out_stride, out_dist, out_dist2;
  FastDiv fd_m, fd_n, fd_nl1;
};

cudaError_t launch_r2r_embed(const R2RDesc& d, int precision, const void* in, void* z,
                             cudaStream_t stream);
cudaError_t launch_r2r_extract(const R2RDesc& d, int precision, const void* F, void* out,
                               cudaStream_t stream);

}  // namespace lfg
