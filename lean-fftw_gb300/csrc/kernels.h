// Launchers of the device kernels (host-callable).
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <vector>

#include "stockham.h"

namespace lfg {

constexpr int kGroupThreads = 256;             // threads per CTA of the group kernels
constexpr size_t kMaxSmemBytes = 232448;       // opt-in shared memory per CTA on sm_103
constexpr size_t kSmemBudget = kMaxSmemBytes - 1024;  // dynamic part planned (static smem aside)

// FP64 group kernel: 2 * C * M * 16 bytes of shared memory.
size_t group_smem_bytes_f64(const GroupDesc& g);
cudaError_t prepare_group_kernels_f64();
cudaError_t launch_group_f64(const GroupDesc& g, bool fwd, const void* in, void* out,
                             cudaStream_t stream);

// FP32 group kernel: 2 * C * M * 8 bytes of shared memory.
cudaError_t prepare_group_kernels_f32();
cudaError_t launch_group_f32(const GroupDesc& g, bool fwd, const void* in, void* out,
                             cudaStream_t stream);

// Persistent FP32 kernel with bulk-async (TMA) prefetch for back-to-back lines of one group
// (input and output 16-byte aligned, C*M even); *status = 1 if a bounded wait gave up.
// give_up (tests of the recovery path): every tile wait gives up at once.  variant: -1 for
// any plan, or stream_variant_f32's index of a power-of-two plan compiled with its passes as
// constants (the same bits, less index arithmetic).
size_t stream_smem_bytes_f32(const GroupDesc& g);
int stream_blocks_per_sm_f32(const GroupDesc& g, int variant = -1);
cudaError_t launch_stream_f32(const GroupDesc& g, bool fwd, const void* in, void* out,
                              int64_t lines, unsigned grid, int* status, cudaStream_t stream,
                              bool give_up = false, int variant = -1);
// Index of the compile-time variant of the persistent binary32 kernel for a one-group plan of
// size n with radices rs, or -1.
int stream_variant_f32(int64_t n, const std::vector<int>& rs);

// One binary64 transform of N <= kClusterMaxN points (one group, contiguous line) on a
// thread-block cluster (the latency path of a lone transform): the lane groups evaluate each
// butterfly level by level of its operation DAG.  build_cluster_image_f64 builds, when the
// plan is made, the device image the kernel copies into shared memory (each pass's geometry,
// its lane-parallel schedule and its twiddle table, from the plan's interleaved tables
// tw_values with per-pass offsets tw_offset in doubles) and fills the launch arguments
// except `img` (the uploaded image), `scale` and `unit` (set at launch); it returns the
// image's bytes, 0 if the group has no cluster form.
constexpr int kClusterMaxN = 4096;
struct ClusterArgs {
  const void* img;
  int img_bytes, N, npass, vwarp, R0, W0, nin0, S;
  double scale;
  int unit;
};
int cluster_size_f64(const GroupDesc& g);
size_t build_cluster_image_f64(const GroupDesc& g, bool fwd, const double* tw_values,
                               const size_t* tw_offset, std::vector<unsigned char>& img,
                               ClusterArgs* args);
size_t cluster_smem_bytes_f64(const ClusterArgs& a);
cudaError_t launch_cluster_f64(const ClusterArgs& a, double scale, const void* in, void* out,
                               cudaStream_t stream);

// Persistent FP32 kernel for tiles of strided sub-problems (three tile buffers: a stage
// filled by asynchronous element copies, two work buffers); in and out 8-byte aligned.
// variant: -1 for any group, or tile_variant_f32's index of a group of a two-group power-of-two
// plan compiled with its passes as constants (the same bits, less index arithmetic).
size_t tile_stream_smem_bytes_f32(const GroupDesc& g, int variant = -1);
int tile_stream_blocks_per_sm_f32(const GroupDesc& g, int variant = -1);
int tile_variant_f32(const GroupDesc& g);
cudaError_t launch_tile_stream_f32(const GroupDesc& g, bool fwd, const void* in, void* out,
                                   unsigned grid, cudaStream_t stream, int variant = -1);

// Register-staged FP32 kernel for a group of two or three passes over contiguous lines (first
// pass from global memory, last pass to global memory, shared tiles between): the first or
// second group of a two-group plan, or the one group of a one-group plan.
// direct_variant_f32 gives the compiled variant of a group (layout, M points, the other
// group's size nsub (1 for one group), compensated twiddles, its radices) or -1.  A second
// group run by it takes its twiddle tables in pass order (not transposed).  The launch checks
// the group's strides against the compiled layout and refuses any other.
enum DirectLayoutKind { kDirectFirstOfTwo = 0, kDirectSecondOfTwo = 1, kDirectSingle = 2 };
int direct_variant_f32(int layout, int M, int nsub, bool comp, const int* radices, int npass);
cudaError_t prepare_direct_kernels_f32();
// The columns of a batch of images (a group whose sub-problems are the columns: line = image,
// in_sub / out_sub = column step, in_elem / out_elem = row step; tiles may straddle images):
// the register-staged kernel of direct_cols_variant_f32 (power-of-two M = 64 .. 512 with
// radices 16.4, 16.8, 16.16, 16.16.2), or -1.
int direct_cols_variant_f32(int M, const int* radices, int npass);
cudaError_t launch_direct_cols_f32(const GroupDesc& g, bool fwd, const void* in, void* out,
                                   int variant, cudaStream_t stream);
cudaError_t launch_direct_f32(const GroupDesc& g, bool fwd, const void* in, void* out,
                              int variant, cudaStream_t stream);

// Batched small transforms on the warp-tile kernel of small.cu (one sub-problem per line):
// one untwiddled pass of R = N <= kSmallMaxN points, binary64 or binary32 (precision 0 / 1),
// or two passes of a binary32 plan of N <= kSmallMaxTwoPassN points with a compiled radix pair.
constexpr int kSmallMaxN = 16;
constexpr int kSmallMaxTwoPassN = 32;
bool small_kernel_applies(const GroupDesc& g, int precision);
cudaError_t prepare_small_kernels();
unsigned small_grid(const GroupDesc& g, int precision);
cudaError_t launch_small(const GroupDesc& g, int precision, bool fwd, const void* in, void* out,
                         unsigned grid, cudaStream_t stream);

// Persistent FP64 kernel over a ragged batch (one launch for all sizes), in kRaggedVariants
// block shapes (threads x minimum CTAs per SM).
constexpr int kRaggedVariants = 5;
// Shared memory: three tile buffers (a stage buffer and two work buffers) of `buf` complex
// elements each.
constexpr size_t ragged_smem_bytes_f64(int64_t buf) { return 3 * (size_t)buf * 16; }
inline bool ragged_tile_fits(int64_t C, int64_t M) {
  return ragged_smem_bytes_f64(tile_elems(C, (int)M)) <= kSmemBudget;
}
// Largest size a ragged batch runs as one pass group (one tile of one transform fits).
inline int64_t ragged_max_single_group() {
  int64_t n = (int64_t)(kSmemBudget / 48);
  while (n > 1 && !ragged_tile_fits(1, n)) --n;
  return n;
}
int ragged_variant_threads(int variant);
int ragged_blocks_per_sm_f64(size_t smem, int variant);
// scratch (optional): grid x slab complex elements of device memory; when given, two-group
// items stage their intermediate there instead of in the output.
cudaError_t launch_ragged_f64(const RaggedLaunch& r, bool fwd, const void* in, void* out,
                              cudaStream_t stream, void* scratch = nullptr, int64_t slab = 0);

}  // namespace lfg
