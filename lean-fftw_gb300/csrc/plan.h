// Host-side plan object and planner of the GB300 execute path.
#pragma once
#include <cuda_runtime.h>

#include <array>
#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "chirp.h"
#include "kernels.h"
#include "generic.h"
#include "pack.h"
#include "r2r.h"
#include "real.h"
#include "stockham.h"

namespace lfg {

enum class Kind { C2C, R2C, C2R, R2R };

// Layout of one side (input or output) of a batched 1-D transform, in complex (C2C) or real
// elements of the side's scalar type, relative to the pointer given at execution.
struct Side {
  int64_t offset = 0;    // element offset of the first element
  int64_t stride = 1;    // between consecutive elements of a line
  int64_t dist = 0;      // between consecutive lines
};

struct Plan;

// One step of a plan that runs through dense buffers: gather (strided -> dense), scatter
// (dense -> strided) or a whole inner plan.  Buffers: 0 the input, 1 the output, 2 and 3 the
// plan's two dense buffers.
struct PackStep {
  enum Op { kGather, kScatter, kPlan } op;
  PackDesc pd{};
  std::shared_ptr<Plan> plan;
  int src = 0, dst = 0;
};

// One axis of a multi-axis complex plan: a 1-D plan along the axis over the other dimensions,
// launched once per entry of `loops` (input and output element offsets of batch dimensions
// beyond the two a launch covers).
struct AxisStage {
  std::shared_ptr<Plan> plan;
  std::vector<std::array<int64_t, 2>> loops;
};

struct Plan {
  Kind kind = Kind::C2C;
  int precision = 0;     // 0: binary64, 1: binary32
  bool fwd = true;
  int64_t n = 0;         // transform size
  int64_t howmany = 1;
  Side in, out;
  // a second (outer) batch dimension of a 1-D complex plan: howmany2 blocks of `howmany`
  // lines, in_dist2 / out_dist2 elements apart
  int64_t howmany2 = 1;
  int64_t in_dist2 = 0, out_dist2 = 0;
  // multi-axis complex plans (rank >= 2, or more vector dimensions than two): the stages run
  // in order, the first from the input to the output, the others in place on the output
  std::vector<AxisStage> stages;
  int64_t in_span = 0;   // spanned input and output, in scalars, from the execution pointer
  int64_t out_span = 0;
  std::vector<int> radices;
  int ngroups = 0;
  GroupDesc groups[2];
  int group_first_pass[2] = {0, 0};
  double flops = 0;      // codelet operations per execution
  // device memory owned by the plan
  int device = 0;
  void* d_twiddles = nullptr;
  mutable void* d_scratch = nullptr;     // intermediate of in-place two-group transforms
  mutable size_t scratch_bytes = 0;
  mutable void* d_host_in = nullptr;     // staging buffers of lfg_execute_host
  mutable void* d_host_out = nullptr;
  bool empty = false;    // a vector dimension of size 0: nothing to do
  int64_t single_max = 0;  // largest size run as one pass group (0: as large as fits)
  bool no_comp = false;    // binary32: no compensated twiddle passes
  int64_t tile = 0;        // complex elements per CTA tile (0: the default)
  bool measure = false;    // LFG_MEASURE: autotune before building
  bool radices_given = false;   // the caller fixed the radix sequence (never reordered)
  // binary32 single-group plans over back-to-back lines run the persistent bulk-copy kernel
  bool stream = false;
  unsigned stream_grid = 0;
  int stream_variant = -1;      // compile-time power-of-two variant of that kernel (-1: none)
  // a lone binary64 transform of at most kClusterMaxN points runs on a thread-block cluster
  bool cluster = false;
  ClusterArgs cluster_args{};   // its launch arguments (cluster_f64.cu)
  void* d_cluster_img = nullptr;   // its device image
  // binary32 groups not covered by the stream kernel: the persistent strided-tile kernel
  // (asynchronous copies of the next tile), one grid per group
  bool tile_stream = false;
  unsigned ts_grid[2] = {0, 0};
  int ts_variant[2] = {-1, -1};  // compile-time two-group power-of-two variants (-1: none)
  // binary32 two-group plans over contiguous lines: the register-staged kernel of each group
  // (direct_f32.cu; -1: none).  Set for both groups or neither; the second group's twiddle
  // tables are then in pass order rather than transposed.
  int direct_variant[2] = {-1, -1};
  unsigned small_grid = 0;      // one-butterfly sizes (N <= 16): the warp-tile kernel's grid
                                // (small.cu; 0: not used)
  unsigned col_ts_grid = 0;     // binary32 column pass of a rank-2 real plan: persistent grid
  int col_direct = -1;          // ... or its register-staged column kernel (-1: none)
  int* d_status = nullptr; // set to 1 on the device when a bounded wait gave up
  bool wait_give_up = false;  // LFG_TEST_WAIT_GIVE_UP: tile waits give up at once (tests)
  bool generic_kernels = false;  // LFG_GENERIC_KERNELS: no compile-time kernel variants
  // real transforms (kind R2C / C2R): rows of the last dimension, and for rank 2 the complex
  // transform along the first dimension (columns of the half spectrum)
  RealDesc real{};
  bool has_col = false;
  GroupDesc col{};
  int64_t col_in_off = 0;        // c2r rank 2: complex offset of the input's first element
  void* d_post = nullptr;
  void* d_col_twiddles = nullptr;
  // real-to-real lines (kind R2R): embedding descriptor, the complex DFT of the embedding
  // size over all lines (none when that size is 1), and the plan's two complex buffers
  // (embedding, spectrum) of lines x M elements each
  R2RDesc r2r{};
  std::shared_ptr<Plan> r2r_dft;
  void* d_r2r_buf = nullptr;
  // complex sizes with a prime factor above 13 (Bluestein): forward and backward transforms
  // of the convolution length L over all lines, two lines x L buffers, chirp and filter
  ChirpDesc chirp{};
  std::shared_ptr<Plan> chirp_fwd, chirp_bwd;
  void* d_chirp_buf = nullptr;
  void* d_chirp_tab = nullptr;
  // small sizes with a prime factor above 13: the generic engine's transform, one CTA a line
  bool generic = false;
  GenericDesc gen{};
  void* d_gen_tab = nullptr;
  // problems the kernels do not take directly (split real/imaginary arrays, strides of either
  // sign, odd, non-smooth or rank >= 3 real transforms) run as a list of steps through two
  // dense complex buffers of pack_elems elements each
  std::vector<PackStep> steps;
  void* d_pack_buf = nullptr;
  int64_t pack_elems = 0;
};

// Geometry of a real transform: vector count `howmany`, rank-2 size n0 x n (rank 1: n0 = 1).
// Real side in doubles, complex side in complex elements; unit stride along the last axis.
struct RealLayout {
  int64_t n0 = 1, n = 0, howmany = 1;
  int64_t r_off = 0, r_bdist = 0, r_rdist = 0;
  int64_t c_off = 0, c_bdist = 0, c_rdist = 0;
};

// Build a real plan (p.kind R2C or C2R, p.fwd set accordingly).  Returns "" on success.
std::string build_real(Plan& p, const RealLayout& L, int64_t tile_target);

// Radix sequence with the fewest codelet operations for size n (first pass untwiddled),
// or an empty vector when n is not 13-smooth.
std::vector<int> choose_radices(int64_t n, int precision);
// Radix sequence of least latency for one transform of size n on a thread-block cluster
// (each pass costs one butterfly's operations per thread plus a fixed pass cost), or empty.
std::vector<int> choose_radices_latency(int64_t n);
// The fewest-operation radices of each factor of the most balanced split n = P * Q (larger
// factor first), so split_point cuts at P; empty if n is prime or not 13-smooth.
std::vector<int> balanced_radices(int64_t n);
// Pass-group split of radix sequence rs for size N (the number of passes in the first group;
// rs.size() = one group; -1 = no split of at most two groups fits): groups of at most
// single_max points (0 = the shared-memory limit), then up to the shared-memory limit, then, if
// may_reorder, after reordering rs around the most balanced factor pair (rs is updated).
int choose_split(int64_t N, std::vector<int>& rs, int64_t single_max, int prec, bool may_reorder);
// Largest binary32 size run as one pass group by default.  Binary32 is bound by HBM, and a
// one-group tile above this size leaves one CTA per SM; larger sizes run two groups of about
// sqrt(n) points each (choose_radices orders the radices for that split).
constexpr int64_t kF32SingleGroupMax = 4096;

// Codelet operation count of a plan's radix sequence, per transform.
double plan_ops(int64_t n, const std::vector<int>& radices);

// Fill groups, tile sizes and twiddle tables of a C2C plan whose size, batch layout and
// radices are set.  Returns an error message, or "" on success.
std::string build_c2c(Plan& p, int64_t tile_target);

// Pass twiddle tables of a radix sequence (host copy; pass 0 has none), with each pass's ns.
struct PassTables {
  std::vector<double> values;
  std::vector<size_t> offset;
  std::vector<int64_t> ns;
};
PassTables make_pass_tables(int64_t N, bool fwd, const std::vector<int>& rs, int precision);
// Store the tables of passes split..end (the second pass group) transposed: within each row
// of ns_g = ns_loc * P values, entry k_loc * P + m moves to m * ns_loc + k_loc, so that the
// threads of a warp, which walk k_loc within one sub-problem m, read consecutive twiddles.
// `comp` marks binary32 passes whose rows come as [hi rows | lo rows] (split_compensated).
void transpose_second_group(PassTables& pt, const std::vector<int>& rs, int split,
                            const std::vector<int>& comp);

bool radix_ok(int R);
std::string check_radices(int64_t N, const std::vector<int>& rs);
int64_t divisor_at_most(int64_t n, int64_t cap);
size_t smem_bytes(int64_t C, int64_t M, int precision);
int64_t max_single_group(int precision);
// Index after the last pass of the first group (rs.size() for a single group), balancing the
// two groups' lengths, both at most max_m; -1 if impossible.
// Store each pass table as (re, im) pairs: row pair (2r, 2r+1) of ns values becomes ns
// pairs, so a butterfly reads each twiddle with one vector load.  Compensated binary32 tables
// interleave their hi and lo halves separately.  Applied after transpose_second_group.
// quads: compensated passes as (hi re, hi im, lo re, lo im) per twiddle instead of a pair table
// of hi values followed by one of lo values.
void interleave_tables(PassTables& pt, const std::vector<int>& rs, const std::vector<int>& comp,
                       bool quads = false);
int split_point(int64_t N, const std::vector<int>& rs, int64_t max_m);
// Fill the passes and tile size of a group covering passes t0..t1-1; tw_base is the device
// copy of PassTables::values.
void fill_group(GroupDesc& g, const std::vector<int>& rs, const PassTables& pt, int t0, int t1,
                int64_t nsub, int64_t tile_target, int precision, const void* tw_base);
void* upload_tables(const std::vector<double>& v, int precision, std::string* err);

void free_plan_memory(Plan& p);

// force_scratch: keep the intermediate of two-group plans in the plan's device scratch even
// out of place (used when `out` is host memory mapped into the device's address space).
// scratch: a caller-supplied device buffer of n * howmany complex elements that takes the
// place of the plan's own scratch for the intermediate of a one-block two-group plan (the
// plan's scratch is then neither allocated nor touched); nullptr = the plan's own.
cudaError_t execute_plan(const Plan& p, const void* in, void* out, cudaStream_t stream,
                         bool force_scratch = false, void* scratch = nullptr);

}  // namespace lfg
