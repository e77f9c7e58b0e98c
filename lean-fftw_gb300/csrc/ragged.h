// Host-side ragged-batch plan (see ragged.cpp).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "plan.h"
#include "stockham.h"

namespace lfg {

struct RaggedOptions {
  int64_t tile_target = 2048;      // complex elements per CTA tile
  int64_t single_max = 2048;       // largest size run as one pass group
  int variant = 0;                 // block shape of the persistent kernel
  std::map<int64_t, std::vector<int>> radices;   // per-size overrides (autotuner)
  // Pass tables by (size, radices), shared by the autotuner's candidate plans of one batch
  // (the exact trigonometric tables dominate a plan's host time); null = no cache.
  std::shared_ptr<std::map<std::pair<int64_t, std::vector<int>>, PassTables>> table_cache;
};

// One launch of the per-size strategy: a batched plan over one size's evenly spaced lines.
struct PerSizeLaunch {
  GroupDesc g[2];
  int ngroups = 1;
  int64_t in_base = 0, out_base = 0;   // complex-element offsets of the first line
};

struct RaggedPlan {
  int precision = 0;
  bool fwd = true;
  int device = 0;
  bool empty = false;
  bool use_graph = true;
  bool per_size_mode = false;
  // per-size launches spread over kPerSizeBranches independent branches (cost-balanced; the
  // launches of one size stay in order on one branch), joined at the end
  bool per_size_concurrent = false;
  std::vector<int> per_size_branch;                    // branch of each per-size launch
  std::vector<cudaStream_t> branch_streams;
  std::vector<cudaEvent_t> branch_events;              // [0]: fork, [1 + b]: join of branch b
  std::vector<int64_t> sizes, in_off, out_off;        // as given (complex elements)
  std::vector<int64_t> line_order;                     // lines sorted by size
  std::vector<int64_t> class_n, class_first, class_count;
  std::vector<std::vector<int>> class_radices;
  std::vector<RaggedClass> classes_host;
  std::vector<RaggedItem> items_host;
  std::vector<PerSizeLaunch> per_size;
  RaggedLaunch launch{};
  int64_t in_span = 0, out_span = 0;                   // complex elements
  bool out_dense = false;                              // outputs tile [0, out_span) exactly
  double flops = 0;
  RaggedOptions options;
  void *d_twiddles = nullptr, *d_classes = nullptr, *d_items = nullptr, *d_in_off = nullptr,
       *d_out_off = nullptr, *d_counter = nullptr;
  mutable void *d_host_in = nullptr, *d_host_out = nullptr;
  mutable void* d_slabs = nullptr;                     // per-CTA intermediates (host-mapped runs)
  mutable size_t slab_bytes = 0;
  mutable cudaGraphExec_t graph_exec = nullptr;
  mutable cudaStream_t capture_stream = nullptr;
  mutable const void* graph_in = nullptr;
  mutable void* graph_out = nullptr;
};

constexpr int kPerSizeBranches = 64;

std::string build_ragged(RaggedPlan& r, const RaggedOptions& opt);
cudaError_t execute_ragged(const RaggedPlan& r, const void* in, void* out, cudaStream_t s);
// Direct launch whose two-group items keep their intermediate in device slabs, so `in` and
// `out` may be host memory mapped into the device's address space.
cudaError_t execute_ragged_mapped(const RaggedPlan& r, const void* in, void* out, cudaStream_t s);
void free_ragged(RaggedPlan& r);

}  // namespace lfg
