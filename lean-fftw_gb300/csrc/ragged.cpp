// Ragged batches: many 1-D complex transforms of different 13-smooth sizes in one launch.
//
// lean-fftw plans and runs one transform at a time (bench/backends/bench-leanfftw.c:270-291);
// its planner measures every candidate schedule per size on the CPU
// (LeanFFTW/Asm/Planner.lean:209-286).  Here a ragged batch is planned once: transforms are
// grouped by size ("classes"), each class gets a radix sequence and a tile shape, and the
// work is cut into items (a tile of same-size transforms, or one whole two-group transform)
// that a persistent kernel pulls from a queue, largest first.  The queue reset and the
// kernel are captured in a CUDA graph and replayed.
//
// Every transform performs the reference passes of its radix sequence, so each output is
// bit-identical to lean-fftw's refTransform for that size and sequence.
#include "ragged.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <map>
#include <numeric>
#include <thread>

#include "generated/opcounts.h"
#include "kernels.h"

namespace lfg {

void free_ragged(RaggedPlan& r) {
  int cur = 0;
  cudaGetDevice(&cur);
  if (cur != r.device) cudaSetDevice(r.device);
  if (r.graph_exec) cudaGraphExecDestroy(r.graph_exec);
  if (r.capture_stream) cudaStreamDestroy(r.capture_stream);
  for (void* p : {r.d_twiddles, r.d_classes, r.d_items, r.d_in_off, r.d_out_off, r.d_counter,
                  r.d_host_in, r.d_host_out, r.d_slabs})
    if (p) cudaFree(p);
  for (cudaStream_t st : r.branch_streams) cudaStreamDestroy(st);
  for (cudaEvent_t ev : r.branch_events) cudaEventDestroy(ev);
  r.branch_streams.clear();
  r.branch_events.clear();
  r.d_slabs = nullptr;
  r.graph_exec = nullptr;
  r.capture_stream = nullptr;
  r.d_twiddles = r.d_classes = r.d_items = r.d_in_off = r.d_out_off = r.d_counter = nullptr;
  r.d_host_in = r.d_host_out = nullptr;
  if (cur != r.device) cudaSetDevice(cur);
}

namespace {

// Butterflies per unit of pass time: a CTA's warp w runs on SM sub-partition w % 4, whose
// FP64 pipe takes a whole warp instruction whatever its active lanes, so a pass of nb
// butterflies keeps the busiest sub-partition for ceil(nb / 128) units of 128 butterflies
// (ceil(nb / 32) warps spread round-robin over 4 sub-partitions).
constexpr int64_t kPassGrain = 4 * 32;
// Fixed cost of one tile (staging the next tile, the store phase, barriers, queue), in
// binary64 operations of pass work: about 9000 per tile of the 8192-size batch on GB300
// (clock64 stamps around each phase of the kernel).
constexpr double kTileOverheadOps = 9000.0;

// Pass time of a tile of C sub-problems of length M through passes t0..t1 of rs, in
// operation-slots (SMSP-granular, see kPassGrain), and the operations it performs.
void tile_lane_cost(int64_t C, int64_t M, const std::vector<int>& rs, int t0, int t1,
                    double* ops, double* slots) {
  for (int t = t0; t < t1; ++t) {
    const int R = rs[t];
    const int64_t nb = C * (M / R);
    const double o = t == 0 ? kOpsUntw[R] : kOpsTw[R];
    *ops += (double)nb * o;
    *slots += (double)(kPassGrain * ((nb + kPassGrain - 1) / kPassGrain)) * o;
  }
}

// Tile width for `total` sub-problems in tiles of at most cmax: the C in [cmax/2, cmax] whose
// tiles (and last, partial tile) take the least modelled time -- pass slots plus the fixed
// cost of each tile; ties to the wider tile.
int64_t lane_efficient_width(int64_t M, const std::vector<int>& rs, int t0, int t1, int64_t total,
                             int64_t cmax) {
  int64_t best = cmax;
  double best_time = -1;
  for (int64_t C = cmax; C >= std::max<int64_t>(1, cmax / 2); --C) {
    double ops = 0, slots = 0;
    const int64_t full = total / C, rem = total % C;
    tile_lane_cost(C, M, rs, t0, t1, &ops, &slots);
    slots = (slots + kTileOverheadOps) * (double)full;
    if (rem) {
      tile_lane_cost(rem, M, rs, t0, t1, &ops, &slots);
      slots += kTileOverheadOps;
    }
    if (best_time < 0 || slots < best_time - 1e-9) {
      best_time = slots;
      best = C;
    }
  }
  return best;
}

}  // namespace

std::string build_ragged(RaggedPlan& r, const RaggedOptions& opt) {
  const int prec = r.precision;
  const int64_t count = (int64_t)r.sizes.size();
  // classes in increasing size; lines sorted by (size, original index)
  std::vector<int64_t> order(count);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(),
                   [&](int64_t a, int64_t b) { return r.sizes[a] < r.sizes[b]; });
  r.line_order = order;
  std::vector<int64_t> in_sorted(count), out_sorted(count);
  for (int64_t i = 0; i < count; ++i) {
    in_sorted[i] = r.in_off[order[i]];
    out_sorted[i] = r.out_off[order[i]];
  }
  // distinct sizes
  r.class_n.clear();
  r.class_first.clear();
  r.class_count.clear();
  for (int64_t i = 0; i < count; ++i) {
    int64_t n = r.sizes[order[i]];
    if (r.class_n.empty() || r.class_n.back() != n) {
      r.class_n.push_back(n);
      r.class_first.push_back(i);
      r.class_count.push_back(0);
    }
    r.class_count.back()++;
  }
  const int ncls = (int)r.class_n.size();
  r.class_radices.assign(ncls, {});
  r.classes_host.assign(ncls, RaggedClass{});

  // radix sequences and twiddle tables of every class, in one device buffer
  std::vector<PassTables> tables(ncls);
  std::vector<size_t> base(ncls, 0);
  std::vector<int> split_c(ncls, 0);
  size_t total = 0;
  r.flops = 0;
  for (int c = 0; c < ncls; ++c) {
    const int64_t n = r.class_n[c];
    auto it = opt.radices.find(n);
    r.class_radices[c] = it != opt.radices.end() ? it->second : choose_radices(n, prec);
    std::string msg = check_radices(n, r.class_radices[c]);
    if (!msg.empty()) return "size " + std::to_string(n) + ": " + msg;
  }
  // the exact trigonometric tables of the distinct sizes, computed on all host threads
  // (independent pure functions of (n, direction, radices)); cached ones are copied
  std::vector<char> cached(ncls, 0);
  if (opt.table_cache)
    for (int c = 0; c < ncls; ++c) {
      auto hit = opt.table_cache->find(std::make_pair(r.class_n[c], r.class_radices[c]));
      if (hit != opt.table_cache->end()) {
        tables[c] = hit->second;
        cached[c] = 1;
      }
    }
  {
    std::atomic<int> next{0};
    std::atomic<bool> failed{false};
    auto work = [&]() {
      try {
        for (int c; (c = next.fetch_add(1)) < ncls;)
          if (!cached[c]) tables[c] = make_pass_tables(r.class_n[c], r.fwd, r.class_radices[c], prec);
      } catch (...) {   // (host allocation) reported below, never thrown across the thread
        failed = true;
        next = ncls;
      }
    };
    const int nthr = (int)std::min<unsigned>(std::max(1u, std::thread::hardware_concurrency()),
                                             (unsigned)std::max(1, ncls / 8));
    std::vector<std::thread> pool;
    for (int i = 1; i < nthr; ++i) {
      try {
        pool.emplace_back(work);
      } catch (...) {   // no more threads: the calling thread does the rest
        break;
      }
    }
    work();
    for (std::thread& t : pool) t.join();
    if (failed) return "host allocation for the twiddle tables failed";
  }
  for (int c = 0; c < ncls; ++c) {
    const int64_t n = r.class_n[c];
    if (opt.table_cache && !cached[c])
      opt.table_cache->emplace(std::make_pair(n, r.class_radices[c]), tables[c]);
    // pass grouping: the per-size strategy splits at the shared-memory limit, the persistent
    // kernel at opt.single_max; the second group's tables are stored transposed
    split_c[c] = split_point(n, r.class_radices[c],
                             r.per_size_mode ? max_single_group(prec)
                                             : std::min(opt.single_max, ragged_max_single_group()));
    if (split_c[c] < 0) return "size " + std::to_string(n) + " needs more than two pass groups";
    transpose_second_group(tables[c], r.class_radices[c], split_c[c], {});
    interleave_tables(tables[c], r.class_radices[c], {});
    base[c] = total;
    total += tables[c].values.size();
    r.flops += plan_ops(n, r.class_radices[c]) * (double)r.class_count[c];
  }
  std::vector<double> all(total);
  for (int c = 0; c < ncls; ++c)
    std::copy(tables[c].values.begin(), tables[c].values.end(), all.begin() + base[c]);
  std::string err;
  r.d_twiddles = upload_tables(all, prec, &err);
  if (!r.d_twiddles) return err;
  const size_t scal = prec == 0 ? sizeof(double) : sizeof(float);

  // groups and work items; the persistent kernel holds three tile buffers of the largest
  // tile (ragged_tile_fits)
  std::vector<RaggedItem> items;
  std::vector<double> item_cost;
  int64_t buf = 0;
  for (int c = 0; c < ncls; ++c) {
    const int64_t n = r.class_n[c];
    const std::vector<int>& rs = r.class_radices[c];
    RaggedClass& rc = r.classes_host[c];
    rc.n = (int)n;
    const void* tw = static_cast<const char*>(r.d_twiddles) + base[c] * scal;
    const int split = split_c[c];
    const double ops_one = plan_ops(n, rs);
    if (split == (int)rs.size()) {
      rc.ngroups = 1;
      GroupDesc& g = rc.g[0];
      fill_group(g, rs, tables[c], 0, (int)rs.size(), 1, opt.tile_target, prec, tw);
      int64_t cmax = std::max<int64_t>(1, opt.tile_target / n);
      while (cmax > 1 && !ragged_tile_fits(cmax, n)) --cmax;
      cmax = std::min<int64_t>(cmax, r.class_count[c]);
      g.C = (int)(r.per_size_mode ? cmax
                                  : lane_efficient_width(n, rs, 0, (int)rs.size(), r.class_count[c], cmax));
      g.in_sub = g.out_sub = 0;
      g.in_elem = g.out_elem = 1;
      g.total_sub = g.C;
      for (int64_t i = 0; i < r.class_count[c]; i += g.C) {
        int cnt = (int)std::min<int64_t>(g.C, r.class_count[c] - i);
        items.push_back(RaggedItem{c, cnt, r.class_first[c] + i});
        item_cost.push_back(ops_one * cnt);
      }
    } else {
      rc.ngroups = 2;
      int64_t P = 1;
      for (int t = 0; t < split; ++t) P *= rs[t];
      const int64_t Q = n / P;
      GroupDesc& g1 = rc.g[0];
      GroupDesc& g2 = rc.g[1];
      fill_group(g1, rs, tables[c], 0, split, Q, opt.tile_target, prec, tw);
      fill_group(g2, rs, tables[c], split, (int)rs.size(), P, opt.tile_target, prec, tw);
      // group 1: x[b + Q i] -> out[b P + m]; group 2: out[i P + m] -> out[o P + m]
      g1.in_sub = 1;
      g1.in_elem = Q;
      g1.out_sub = P;
      g1.out_elem = 1;
      g2.in_sub = 1;
      g2.in_elem = P;
      g2.out_sub = 1;
      g2.out_elem = P;
      g1.total_sub = Q;
      g2.total_sub = P;
      if (!r.per_size_mode) {   // tile widths with the least modelled pass time
        for (GroupDesc* g : {&g1, &g2}) {
          int64_t cmax = std::max<int64_t>(1, opt.tile_target / g->M);
          while (cmax > 1 && !ragged_tile_fits(cmax, g->M)) --cmax;
          cmax = std::min<int64_t>(cmax, g->nsub);
          const int t0 = g == &g1 ? 0 : split, t1 = g == &g1 ? split : (int)rs.size();
          g->C = (int)lane_efficient_width(g->M, rs, t0, t1, g->nsub, cmax);
        }
      }
      for (int64_t i = 0; i < r.class_count[c]; ++i) {
        items.push_back(RaggedItem{c, 1, r.class_first[c] + i});
        item_cost.push_back(ops_one);
      }
    }
    for (int gi = 0; gi < rc.ngroups; ++gi) {
      GroupDesc& g = rc.g[gi];
      while (g.C > 1 && !ragged_tile_fits(g.C, g.M)) --g.C;
      buf = std::max<int64_t>(buf, tile_elems(g.C, g.M));
    }
  }
  // largest items first
  std::vector<size_t> perm(items.size());
  std::iota(perm.begin(), perm.end(), 0);
  std::stable_sort(perm.begin(), perm.end(), [&](size_t a, size_t b) { return item_cost[a] > item_cost[b]; });
  r.items_host.resize(items.size());
  for (size_t i = 0; i < perm.size(); ++i) r.items_host[i] = items[perm[i]];

  // device copies
  auto up = [&](void** d, const void* h, size_t bytes) -> bool {
    if (cudaMalloc(d, std::max<size_t>(bytes, 16)) != cudaSuccess) return false;
    return bytes == 0 || cudaMemcpy(*d, h, bytes, cudaMemcpyHostToDevice) == cudaSuccess;
  };
  for (RaggedClass& rc : r.classes_host)
    for (int gi = 0; gi < rc.ngroups; ++gi) set_divisors(rc.g[gi]);
  if (!up(&r.d_classes, r.classes_host.data(), r.classes_host.size() * sizeof(RaggedClass)) ||
      !up(&r.d_items, r.items_host.data(), r.items_host.size() * sizeof(RaggedItem)) ||
      !up(&r.d_in_off, in_sorted.data(), in_sorted.size() * sizeof(int64_t)) ||
      !up(&r.d_out_off, out_sorted.data(), out_sorted.size() * sizeof(int64_t)) ||
      cudaMalloc(&r.d_counter, 256) != cudaSuccess)
    return "device allocation for the ragged plan failed";
  cudaMemset(r.d_counter, 0, 256);

  cudaDeviceProp prop;
  cudaGetDeviceProperties(&prop, r.device);
  r.launch.classes = static_cast<const RaggedClass*>(r.d_classes);
  r.launch.items = static_cast<const RaggedItem*>(r.d_items);
  r.launch.nitems = (int)r.items_host.size();
  r.launch.in_off = static_cast<const int64_t*>(r.d_in_off);
  r.launch.out_off = static_cast<const int64_t*>(r.d_out_off);
  r.launch.counter = static_cast<unsigned*>(r.d_counter);
  r.launch.buf = (int)buf;
  r.launch.smem = ragged_smem_bytes_f64(buf);
  const size_t smem = r.launch.smem;
  r.launch.variant = opt.variant;
  const int per_sm = prec == 0 ? ragged_blocks_per_sm_f64(smem, opt.variant) : 1;
  const int64_t want = (int64_t)prop.multiProcessorCount * per_sm;
  r.launch.grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)r.items_host.size()));

  // per-size strategy (the comparison point): one batched launch per distinct size when the
  // class's lines are evenly spaced in both buffers, else one launch per transform
  r.per_size.clear();
  for (int c = 0; c < ncls; ++c) {
    const int64_t n = r.class_n[c];
    const int64_t f = r.class_first[c], k = r.class_count[c];
    bool even = true;
    int64_t din = k > 1 ? in_sorted[f + 1] - in_sorted[f] : n;
    int64_t dout = k > 1 ? out_sorted[f + 1] - out_sorted[f] : n;
    for (int64_t i = 1; i < k && even; ++i)
      even = in_sorted[f + i] - in_sorted[f + i - 1] == din && out_sorted[f + i] - out_sorted[f + i - 1] == dout;
    even = even && din > 0 && dout > 0;
    const std::vector<int>& rs = r.class_radices[c];
    const void* tw = static_cast<const char*>(r.d_twiddles) + base[c] * scal;
    const int64_t lines = even ? k : 1;
    for (int64_t i = 0; i < (even ? 1 : k); ++i) {
      PerSizeLaunch L;
      L.in_base = in_sorted[f + i];
      L.out_base = out_sorted[f + i];
      const int split = split_c[c];
      if (split == (int)rs.size()) {
        L.ngroups = 1;
        GroupDesc& g = L.g[0];
        fill_group(g, rs, tables[c], 0, (int)rs.size(), 1, opt.tile_target, prec, tw);
        int64_t cmax = std::max<int64_t>(1, opt.tile_target / n);
        while (cmax > 1 && smem_bytes(cmax, n, prec) > kSmemBudget) --cmax;
        g.C = (int)std::min<int64_t>(cmax, lines);
        g.total_sub = lines;
        g.in_line = din;
        g.out_line = dout;
        g.in_sub = g.out_sub = 0;
        g.in_elem = g.out_elem = 1;
      } else {
        L.ngroups = 2;
        int64_t P = 1;
        for (int t = 0; t < split; ++t) P *= rs[t];
        const int64_t Q = n / P;
        fill_group(L.g[0], rs, tables[c], 0, split, Q, opt.tile_target, prec, tw);
        fill_group(L.g[1], rs, tables[c], split, (int)rs.size(), P, opt.tile_target, prec, tw);
        L.g[0].total_sub = lines * Q;
        L.g[1].total_sub = lines * P;
        L.g[0].in_line = din;
        L.g[0].in_sub = 1;
        L.g[0].in_elem = Q;
        L.g[0].out_line = dout;
        L.g[0].out_sub = P;
        L.g[0].out_elem = 1;
        L.g[1].in_line = dout;
        L.g[1].in_sub = 1;
        L.g[1].in_elem = P;
        L.g[1].out_line = dout;
        L.g[1].out_sub = 1;
        L.g[1].out_elem = P;
      }
      r.per_size.push_back(L);
    }
  }
  if (r.per_size_mode && r.per_size_concurrent) {
    // longest-processing-time assignment of the launches to the branches
    std::vector<double> cost(r.per_size.size());
    for (size_t i = 0; i < r.per_size.size(); ++i) {
      const PerSizeLaunch& L = r.per_size[i];
      const int64_t n = L.ngroups == 1 ? (int64_t)L.g[0].M : (int64_t)L.g[0].M * L.g[1].M;
      const int64_t lines = L.ngroups == 1 ? L.g[0].total_sub : L.g[0].total_sub / std::max(1, L.g[0].nsub);
      cost[i] = (double)n * (double)lines * std::log2((double)std::max<int64_t>(2, n));
    }
    std::vector<size_t> ord(cost.size());
    std::iota(ord.begin(), ord.end(), 0);
    std::stable_sort(ord.begin(), ord.end(), [&](size_t a, size_t b) { return cost[a] > cost[b]; });
    std::vector<double> load(kPerSizeBranches, 0.0);
    r.per_size_branch.assign(r.per_size.size(), 0);
    for (size_t i : ord) {
      const int b = (int)(std::min_element(load.begin(), load.end()) - load.begin());
      r.per_size_branch[i] = b;
      load[b] += cost[i];
    }
    for (int b = 0; b < kPerSizeBranches; ++b) {
      cudaStream_t st = nullptr;
      if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess)
        return "stream creation for the per-size branches failed";
      r.branch_streams.push_back(st);
    }
    for (int b = 0; b <= kPerSizeBranches; ++b) {
      cudaEvent_t ev = nullptr;
      if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess)
        return "event creation for the per-size branches failed";
      r.branch_events.push_back(ev);
    }
  }
  return "";
}

cudaError_t execute_ragged_direct(const RaggedPlan& r, const void* in, void* out, cudaStream_t s) {
  if (r.per_size_mode) {
    const size_t es = r.precision == 0 ? 16 : 8;
    const bool conc = r.per_size_concurrent && !r.branch_streams.empty();
    cudaError_t e = cudaSuccess;
    if (conc) {
      // fork: every branch starts after the work already queued on s
      e = cudaEventRecord(r.branch_events[0], s);
      for (size_t b = 0; b < r.branch_streams.size() && e == cudaSuccess; ++b)
        e = cudaStreamWaitEvent(r.branch_streams[b], r.branch_events[0], 0);
    }
    for (size_t i = 0; i < r.per_size.size() && e == cudaSuccess; ++i) {
      const PerSizeLaunch& L = r.per_size[i];
      cudaStream_t st = conc ? r.branch_streams[r.per_size_branch[i]] : s;
      const char* ib = static_cast<const char*>(in) + L.in_base * es;
      char* ob = static_cast<char*>(out) + L.out_base * es;
      for (int gi = 0; gi < L.ngroups && e == cudaSuccess; ++gi)
        e = launch_group_f64(L.g[gi], r.fwd, gi == 0 ? (const void*)ib : (const void*)ob, ob, st);
    }
    if (conc) {
      // join: s continues after every branch (also on an error, so no branch is left open
      // in a capture)
      for (size_t b = 0; b < r.branch_streams.size(); ++b) {
        cudaError_t e1 = cudaEventRecord(r.branch_events[1 + b], r.branch_streams[b]);
        if (e1 == cudaSuccess) e1 = cudaStreamWaitEvent(s, r.branch_events[1 + b], 0);
        if (e == cudaSuccess) e = e1;
      }
    }
    return e;
  }
  cudaError_t e = cudaMemsetAsync(r.d_counter, 0, sizeof(unsigned), s);
  if (e != cudaSuccess) return e;
  return launch_ragged_f64(r.launch, r.fwd, in, out, s);
}

cudaError_t execute_ragged_mapped(const RaggedPlan& r, const void* in, void* out, cudaStream_t s) {
  // the largest two-group size sets the slab of each persistent CTA
  int64_t slab = 0;
  for (size_t c = 0; c < r.classes_host.size(); ++c)
    if (r.classes_host[c].ngroups == 2) slab = std::max<int64_t>(slab, r.class_n[c]);
  const size_t need = (size_t)slab * r.launch.grid * (r.precision == 0 ? 16 : 8);
  if (need > r.slab_bytes) {
    if (r.d_slabs) cudaFree(r.d_slabs);
    r.d_slabs = nullptr;
    r.slab_bytes = 0;
    cudaError_t e = cudaMalloc(&r.d_slabs, need);
    if (e != cudaSuccess) return e;
    r.slab_bytes = need;
  }
  cudaError_t e = cudaMemsetAsync(r.d_counter, 0, sizeof(unsigned), s);
  if (e != cudaSuccess) return e;
  return launch_ragged_f64(r.launch, r.fwd, in, out, s, slab ? r.d_slabs : nullptr, slab);
}

cudaError_t execute_ragged(const RaggedPlan& r, const void* in, void* out, cudaStream_t s) {
  if (r.empty) return cudaSuccess;
  if (!r.use_graph) return execute_ragged_direct(r, in, out, s);
  if (!r.graph_exec || r.graph_in != in || r.graph_out != out) {
    // capture the queue reset and the launch(es) on a private stream, then replay
    if (r.graph_exec) {
      cudaGraphExecDestroy(r.graph_exec);
      r.graph_exec = nullptr;
    }
    if (!r.capture_stream) {
      cudaError_t e = cudaStreamCreateWithFlags(&r.capture_stream, cudaStreamNonBlocking);
      if (e != cudaSuccess) return e;
    }
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamBeginCapture(r.capture_stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return e;
    cudaError_t e2 = execute_ragged_direct(r, in, out, r.capture_stream);
    e = cudaStreamEndCapture(r.capture_stream, &graph);
    if (e2 != cudaSuccess) {
      if (graph) cudaGraphDestroy(graph);
      return e2;
    }
    if (e != cudaSuccess) return e;
    e = cudaGraphInstantiate(&r.graph_exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return e;
    r.graph_in = in;
    r.graph_out = out;
  }
  return cudaGraphLaunch(r.graph_exec, s);
}

}  // namespace lfg
