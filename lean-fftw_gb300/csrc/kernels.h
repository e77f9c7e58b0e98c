// Launchers of the device kernels (host-callable).
#pragma once
#include <cuda_runtime.h>

#include <cstddef>

#include "stockham.h"

namespace lfg {

constexpr int kGroupThreads = 256;             // threads per CTA of the group kernels
constexpr size_t kMaxSmemBytes = 232448;       // opt-in shared memory per CTA on sm_103

// FP64 group kernel: 2 * C * M * 16 bytes of shared memory.
size_t group_smem_bytes_f64(const GroupDesc& g);
cudaError_t prepare_group_kernels_f64();
cudaError_t launch_group_f64(const GroupDesc& g, bool fwd, const void* in, void* out,
                             cudaStream_t stream);

}  // namespace lfg
