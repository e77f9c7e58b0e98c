// The generic engine's mixed-radix transform for sizes with a prime factor above 13
// (generic.cu): descriptor and launcher.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace lfg {

constexpr int kGenericMaxN = 4096;   // one line per CTA, two buffers in shared memory

// Lines l = l1 + nl1 * l2 (l1 < nl1): input at l1*in_dist + l2*in_dist2, element stride
// in_stride (complex elements, from the pointer given), likewise for the output.
struct GenericDesc {
  int n, nf;
  int f[24];       // prime factors, ascending (lean-fftw `primeFactors`)
  int ni[24];      // ni[i] = f[i] * ... * f[nf-1]
  int64_t lines, nl1;
  int64_t in_stride, in_dist, in_dist2;
  int64_t out_stride, out_dist, out_dist2;
  double scale;    // outputs multiplied by this on store unless it is exactly 1
  const void* tab; // cos/sin(2 pi m / n), m < n, in the plan's precision
};

cudaError_t prepare_generic_kernels();
cudaError_t launch_generic(const GenericDesc& d, int precision, bool fwd, const void* in, void* out,
                           cudaStream_t stream);

}  // namespace lfg
