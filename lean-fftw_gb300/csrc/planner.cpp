// Planner of the GB300 execute path: radix choice, pass grouping, twiddle tables.
//
// lean-fftw's planner (LeanFFTW/Asm/Planner.lean:84-286) enumerates radix sequences and
// schedules, prunes them by proved operation counts (`raceOrder`, :196-205) and times the
// survivors on the CPU.  On GB300 the binary64 path is bound by the FP64 pipe, so the
// operation count of the codelets is the dominant cost: LFG_ESTIMATE picks the sequence
// with the fewest codelet operations directly (a dynamic program over the divisors of n),
// and LFG_MEASURE (api.cpp) times the leading candidates on the device.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <map>

#include "generated/opcounts.h"
#include "generated/wide_f64.h"
#include "kernels.h"
#include "plan.h"
#include "real.h"
#include "trig.h"

namespace lfg {
namespace {

}  // namespace

bool radix_ok(int R) { return R >= 2 && R <= kMaxRadix && kOpsUntw[R] > 0; }

// LFG_DIRECT=0 in the environment (read at planning): binary32 plans use the copy-staged
// kernels instead of the register-staged ones (for comparisons; the same bits).
static bool direct_enabled() {
  const char* s = std::getenv("LFG_DIRECT");
  return !(s && s[0] == '0');
}

// LFG_SMALL=0 in the environment (read at planning): one-butterfly sizes run on the group or
// bulk-copy kernels instead of the warp-tile kernel (for comparisons; the same bits).
static bool small_enabled() {
  const char* s = std::getenv("LFG_SMALL");
  return !(s && s[0] == '0');
}

// Where the warp-tile kernel runs a plan it has a variant for, from 1 GiB batches on GB300:
// binary64 one-butterfly sizes, every N (1.04-2.2x the group kernel); binary32 one-butterfly
// sizes, every N except, where the persistent bulk-copy kernel takes the plan (back-to-back
// lines, N even), N = 2, 4 and 12, which that kernel runs at 0.92-0.98 of HBM against
// 0.89-0.98 (N = 6 and 10: 0.92-0.93 against 0.86-0.87); binary32 two-pass sizes only where the
// bulk-copy kernel does not run (odd N or other layouts: N = 21, 25, 27 take 0.45-0.56 ms
// against 0.76-0.78 on the group kernel, while the bulk-copy kernel runs the even sizes faster,
// N = 32 in 0.47 ms against 0.68).
static bool small_preferred(int prec, int64_t N, int npass, bool bulk_copy) {
  if (prec == 0) return true;
  if (npass == 2) return !bulk_copy;
  return !(bulk_copy && (N == 2 || N == 4 || N == 12));
}

namespace {

// per-point operations of a twiddled pass of radix R
double tw_cost(int R) { return (double)kOpsTw[R] / R; }
double untw_cost(int R) { return (double)kOpsUntw[R] / R; }

struct Best {
  double cost;
  std::vector<int> seq;
};

// Cheapest sequence of twiddled radices with product m (per point), memoised.
const Best& best_tail(int64_t m, std::map<int64_t, Best>& memo) {
  auto it = memo.find(m);
  if (it != memo.end()) return it->second;
  Best b{INFINITY, {}};
  if (m == 1) {
    b.cost = 0;
  } else {
    for (int R = kMaxRadix; R >= 2; --R) {
      if (!radix_ok(R) || m % R) continue;
      const Best& t = best_tail(m / R, memo);
      if (!std::isfinite(t.cost)) continue;
      double c = tw_cost(R) + t.cost;
      // fewer operations first; on a tie, fewer passes
      if (c < b.cost - 1e-12 || (std::fabs(c - b.cost) <= 1e-12 && t.seq.size() + 1 < b.seq.size())) {
        b.cost = c;
        b.seq = t.seq;
        b.seq.insert(b.seq.begin(), R);
      }
    }
  }
  return memo[m] = b;
}

}  // namespace

// Largest divisor of n that is <= cap (at least 1).
int64_t divisor_at_most(int64_t n, int64_t cap) {
  if (cap >= n) return n;
  for (int64_t d = cap; d >= 1; --d)
    if (n % d == 0) return d;
  return 1;
}

size_t smem_bytes(int64_t C, int64_t M, int precision) {
  // two tile buffers of C sub-problems, sub_pitch(M) elements apart (stockham.h)
  return 2 * (size_t)tile_elems(C, (int)M) * (precision == 0 ? 16 : 8);
}

std::vector<int> balanced_radices(int64_t n) {
  int64_t bestP = 0;
  double bestd = INFINITY;
  for (int64_t P = 2; P * P <= n; ++P) {
    if (n % P) continue;
    const double d = std::fabs(std::log((double)P) - std::log((double)(n / P)));
    if (d < bestd) {
      bestd = d;
      bestP = P;
    }
  }
  if (bestP == 0) return {};
  std::vector<int> a = choose_radices(n / bestP, 0), b = choose_radices(bestP, 0);
  if (a.empty() || b.empty()) return {};
  a.insert(a.end(), b.begin(), b.end());
  return a;
}

std::vector<int> choose_radices(int64_t n, int precision) {
  if (n < 2) return {};
  if (precision == 1 && n > kF32SingleGroupMax) {
    // binary32 two-group sizes: both groups get tiles of ~sqrt(n) points
    std::vector<int> b = balanced_radices(n);
    if (!b.empty()) return b;
  }
  std::map<int64_t, Best> memo;
  double best = INFINITY;
  std::vector<int> seq;
  for (int R0 = kMaxRadix; R0 >= 2; --R0) {
    if (!radix_ok(R0) || n % R0) continue;
    const Best& t = best_tail(n / R0, memo);
    if (!std::isfinite(t.cost)) continue;
    double c = untw_cost(R0) + t.cost;
    if (c < best - 1e-12 || (std::fabs(c - best) <= 1e-12 && t.seq.size() + 1 < seq.size())) {
      best = c;
      seq = t.seq;
      seq.insert(seq.begin(), R0);
    }
  }
  return seq;
}

std::vector<int> choose_radices_latency(int64_t n) {
  // a lone transform runs on a thread-block cluster whose lane groups evaluate each butterfly
  // level by level of its operation DAG (cluster_f64.cu): a pass costs its schedule's depth
  // times the rounds its butterflies need on the cluster's 2048 lanes (sixteen CTAs of 128
  // threads), plus a fixed cost per pass -- input loads, distributed stores, the cluster
  // barrier -- of kPassFixed levels
  constexpr double kPassFixed = 5.0;
  constexpr int64_t kLanes = 2048;
  if (n < 2) return {};
  auto pass_cost = [&](int R, bool tw) {
    const WideInfo& w = kWideInfo[1][R][tw ? 1 : 0];
    const int64_t rounds = ((n / R) * w.W + kLanes - 1) / kLanes;
    return (double)(rounds * w.depth) + kPassFixed;
  };
  std::map<int64_t, std::pair<double, std::vector<int>>> memo;   // twiddled tail of length m
  std::function<const std::pair<double, std::vector<int>>&(int64_t)> tail =
      [&](int64_t m) -> const std::pair<double, std::vector<int>>& {
    auto it = memo.find(m);
    if (it != memo.end()) return it->second;
    std::pair<double, std::vector<int>> best{m == 1 ? 0.0 : INFINITY, {}};
    if (m > 1)
      for (int R = kMaxRadix; R >= 2; --R) {
        if (!radix_ok(R) || m % R) continue;
        const auto& t = tail(m / R);
        if (!std::isfinite(t.first)) continue;
        const double c = pass_cost(R, true) + t.first;
        if (c < best.first - 1e-12) {
          best.first = c;
          best.second = t.second;
          best.second.insert(best.second.begin(), R);
        }
      }
    return memo.emplace(m, best).first->second;
  };
  double best = INFINITY;
  std::vector<int> seq;
  for (int R0 = kMaxRadix; R0 >= 2; --R0) {
    if (!radix_ok(R0) || n % R0) continue;
    const auto& t = tail(n / R0);
    if (!std::isfinite(t.first)) continue;
    const double c = pass_cost(R0, false) + t.first;
    if (c < best - 1e-12) {
      best = c;
      seq = t.second;
      seq.insert(seq.begin(), R0);
    }
  }
  return seq;
}

double plan_ops(int64_t n, const std::vector<int>& rs) {
  double ops = 0;
  for (size_t t = 0; t < rs.size(); ++t)
    ops += (double)(n / rs[t]) * (t == 0 ? kOpsUntw[rs[t]] : kOpsTw[rs[t]]);
  return ops;
}

void free_plan_memory(Plan& p) {
  int cur = 0;
  cudaGetDevice(&cur);
  if (cur != p.device) cudaSetDevice(p.device);
  if (p.d_twiddles) cudaFree(p.d_twiddles);
  if (p.d_scratch) cudaFree(p.d_scratch);
  if (p.d_host_in) cudaFree(p.d_host_in);
  if (p.d_host_out) cudaFree(p.d_host_out);
  if (p.d_post) cudaFree(p.d_post);
  if (p.d_col_twiddles) cudaFree(p.d_col_twiddles);
  if (p.d_status) cudaFree(p.d_status);
  if (p.d_r2r_buf) cudaFree(p.d_r2r_buf);
  if (p.d_gen_tab) cudaFree(p.d_gen_tab);
  p.d_gen_tab = nullptr;
  if (p.d_cluster_img) cudaFree(p.d_cluster_img);
  p.d_cluster_img = nullptr;
  p.cluster = false;
  if (p.d_pack_buf) cudaFree(p.d_pack_buf);
  p.d_pack_buf = nullptr;
  for (PackStep& st : p.steps)
    if (st.plan) free_plan_memory(*st.plan);
  p.steps.clear();
  if (p.d_chirp_buf) cudaFree(p.d_chirp_buf);
  if (p.d_chirp_tab) cudaFree(p.d_chirp_tab);
  if (p.chirp_fwd) free_plan_memory(*p.chirp_fwd);
  if (p.chirp_bwd) free_plan_memory(*p.chirp_bwd);
  p.chirp_fwd.reset();
  p.chirp_bwd.reset();
  p.d_chirp_buf = p.d_chirp_tab = nullptr;
  if (p.r2r_dft) free_plan_memory(*p.r2r_dft);
  p.r2r_dft.reset();
  p.d_r2r_buf = nullptr;
  p.d_status = nullptr;
  p.d_twiddles = p.d_scratch = p.d_host_in = p.d_host_out = nullptr;
  p.d_post = p.d_col_twiddles = nullptr;
  for (AxisStage& s : p.stages)
    if (s.plan) free_plan_memory(*s.plan);
  p.stages.clear();
  if (cur != p.device) cudaSetDevice(cur);
}

PassTables make_pass_tables(int64_t N, bool fwd, const std::vector<int>& rs, int precision) {
  PassTables pt;
  std::vector<double> tab = cos_sin_2pi_table((uint64_t)N);
  pt.offset.assign(rs.size(), 0);
  pt.ns.assign(rs.size(), 0);
  size_t total = 0;
  int64_t acc = 1;
  for (size_t t = 0; t < rs.size(); ++t) {
    pt.ns[t] = acc;
    acc *= rs[t];
    if (t == 0) continue;
    pt.offset[t] = total;
    total += 2 * (size_t)(rs[t] - 1) * pt.ns[t];
    total = (total + 3) & ~(size_t)3;   // 32-byte aligned tables
  }
  pt.values.assign(total, 0.0);
  for (size_t t = 1; t < rs.size(); ++t)
    pass_twiddles(tab, fwd, (uint64_t)N, rs[t], (uint64_t)pt.ns[t], pt.values.data() + pt.offset[t]);
  (void)precision;
  return pt;
}

void transpose_second_group(PassTables& pt, const std::vector<int>& rs, int split,
                            const std::vector<int>& comp) {
  if (split <= 0 || split >= (int)rs.size()) return;
  int64_t P = 1;
  for (int t = 0; t < split; ++t) P *= rs[t];
  std::vector<double> row;
  for (int t = split; t < (int)rs.size(); ++t) {
    if (t == 0) continue;
    const int64_t ns = pt.ns[t], nl = ns / P;
    const int rows = 2 * (rs[t] - 1) * (!comp.empty() && comp[t] ? 2 : 1);
    row.resize((size_t)ns);
    for (int q = 0; q < rows; ++q) {
      double* v = pt.values.data() + pt.offset[t] + (size_t)q * ns;
      for (int64_t k = 0; k < nl; ++k)
        for (int64_t m = 0; m < P; ++m) row[(size_t)(m * nl + k)] = v[k * P + m];
      std::copy(row.begin(), row.end(), v);
    }
  }
}

void interleave_tables(PassTables& pt, const std::vector<int>& rs, const std::vector<int>& comp,
                       bool quads) {
  std::vector<double> pairs;
  for (size_t t = 1; t < rs.size(); ++t) {
    const int64_t ns = pt.ns[t];
    if (quads && !comp.empty() && comp[t]) {
      // (hi re, hi im, lo re, lo im) per twiddle: one 16-byte load in binary32
      double* v = pt.values.data() + pt.offset[t];
      const size_t len = 2 * (size_t)(rs[t] - 1) * ns;   // one part
      pairs.assign(v, v + 2 * len);
      for (int r = 0; r < rs[t] - 1; ++r)
        for (int64_t k = 0; k < ns; ++k) {
          double* q = v + 4 * ((size_t)r * ns + k);
          q[0] = pairs[(size_t)(2 * r) * ns + k];
          q[1] = pairs[(size_t)(2 * r + 1) * ns + k];
          q[2] = pairs[len + (size_t)(2 * r) * ns + k];
          q[3] = pairs[len + (size_t)(2 * r + 1) * ns + k];
        }
      continue;
    }
    const int parts = !comp.empty() && comp[t] ? 2 : 1;   // hi table, then lo table
    for (int part = 0; part < parts; ++part) {
      double* v = pt.values.data() + pt.offset[t] + (size_t)part * 2 * (rs[t] - 1) * ns;
      pairs.assign(v, v + 2 * (size_t)(rs[t] - 1) * ns);
      for (int r = 0; r < rs[t] - 1; ++r)
        for (int64_t k = 0; k < ns; ++k) {
          v[2 * ((size_t)r * ns + k)] = pairs[(size_t)(2 * r) * ns + k];
          v[2 * ((size_t)r * ns + k) + 1] = pairs[(size_t)(2 * r + 1) * ns + k];
        }
    }
  }
}

int split_point(int64_t N, const std::vector<int>& rs, int64_t max_m) {
  if (N <= max_m) return (int)rs.size();
  int best = -1;
  int64_t bestv = INT64_MAX;
  int64_t P = 1;
  for (int t = 0; t + 1 < (int)rs.size(); ++t) {
    P *= rs[t];
    int64_t Q = N / P;
    if (P > max_m || Q > max_m) continue;
    int64_t v = std::max(P, Q);
    if (v < bestv) { bestv = v; best = t + 1; }
  }
  return best;
}

void fill_group(GroupDesc& g, const std::vector<int>& rs, const PassTables& pt, int t0, int t1,
                int64_t nsub, int64_t tile_target, int precision, const void* tw_base) {
  int64_t M = 1;
  for (int t = t0; t < t1; ++t) M *= rs[t];
  g.M = (int)M;
  g.npass = t1 - t0;
  g.nsub = (int)nsub;
  int64_t cmax = std::max<int64_t>(1, tile_target / M);
  // strided sub-problems are copied as runs of C neighbouring elements: keep the binary32
  // runs at 64 bytes or more (two 32-byte sectors), which HBM serves at full rate
  if (precision == 1 && nsub > 1) cmax = std::max<int64_t>(cmax, 8);
  while (cmax > 1 && smem_bytes(cmax, M, precision) > kSmemBudget) --cmax;
  // tiles may straddle lines (the sub-problem index is taken per element), so C need not
  // divide nsub; prefer a divisor when one is close to the target
  const int64_t dv = divisor_at_most(nsub, cmax);
  g.C = (int)(2 * dv >= cmax ? dv : cmax);
  int64_t P0 = 1;
  for (int t = 0; t < t0; ++t) P0 *= rs[t];
  g.kmul = (int)P0;
  g.twsub = t0 > 0 ? 1 : 0;
  g.scale = 1.0;
  for (int t = 0; t < kMaxPass; ++t) g.pass[t].comp = 0;
  for (int t = t0; t < t1; ++t) {
    PassDesc& d = g.pass[t - t0];
    d.R = rs[t];
    d.ns_g = (int)pt.ns[t];
    d.ns_loc = (int)(pt.ns[t] / P0);
    if (t == 0) d.tw = nullptr;
    else if (precision == 0) d.tw = (const double*)tw_base + pt.offset[t];
    else d.tw = (const float*)tw_base + pt.offset[t];
  }
}

std::string check_radices(int64_t N, const std::vector<int>& rs) {
  if (rs.empty()) return "no radix sequence";
  if ((int)rs.size() > kMaxPass) return "too many passes";
  int64_t prod = 1;
  for (int R : rs) {
    if (!radix_ok(R)) return "radix " + std::to_string(R) + " has no codelet";
    prod *= R;
  }
  if (prod != N) return "radices do not multiply to n";
  return "";
}

void* upload_tables(const std::vector<double>& v, int precision, std::string* err) {
  void* d = nullptr;
  size_t bytes;
  std::vector<float> v32;
  const void* src;
  if (precision == 0) {
    bytes = std::max<size_t>(v.size(), 4) * sizeof(double);
    src = v.data();
  } else {
    v32.assign(v.begin(), v.end());
    v32.resize(std::max<size_t>(v32.size(), 4));
    bytes = v32.size() * sizeof(float);
    src = v32.data();
  }
  if (cudaMalloc(&d, bytes) != cudaSuccess) {
    *err = "cudaMalloc of twiddle tables failed";
    return nullptr;
  }
  if (!v.empty()) {
    cudaError_t e = cudaMemcpy(d, src, std::min(bytes, (precision == 0 ? 8 : 4) * v.size()),
                               cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
      *err = std::string("twiddle upload: ") + cudaGetErrorString(e);
      cudaFree(d);
      return nullptr;
    }
  }
  return d;
}

int64_t max_single_group(int precision) {
  // largest n with two padded tile buffers within the budget
  const int64_t es = precision == 0 ? 16 : 8;
  int64_t n = (int64_t)(kSmemBudget / (2 * es));
  while (n > 1 && smem_bytes(1, n, precision) > kSmemBudget) --n;
  return n;
}

// binary32 plans of size >= 2^16 multiply by compensated (hi, lo) twiddles in their last
// passes (the second group's, or the last two of a single group)
std::vector<int> compensated_passes(int64_t N, const std::vector<int>& rs, int split, int precision) {
  std::vector<int> comp(rs.size(), 0);
  if (precision != 1 || N < (1 << 16)) return comp;
  const int first = split < (int)rs.size() ? split : std::max(1, (int)rs.size() - 2);
  for (int t = std::max(first, 1); t < (int)rs.size(); ++t) comp[t] = 1;
  return comp;
}

// Re-lay the tables of compensated passes as [hi table | lo table] (binary32 parts of each
// binary64 value: hi = fl32(v), lo = fl32(v - hi)); other tables stay binary64 and are rounded
// on upload.  Returns the new table array, in binary64 scalars holding binary32-exact values.
std::vector<double> split_compensated(PassTables& pt, const std::vector<int>& rs,
                                      const std::vector<int>& comp) {
  std::vector<double> out;
  std::vector<size_t> off(rs.size(), 0);
  for (size_t t = 1; t < rs.size(); ++t) {
    const size_t len = 2 * (size_t)(rs[t] - 1) * pt.ns[t];
    off[t] = out.size();
    const double* v = pt.values.data() + pt.offset[t];
    if (comp[t]) {
      for (size_t i = 0; i < len; ++i) out.push_back((double)(float)v[i]);
      for (size_t i = 0; i < len; ++i) out.push_back((double)(float)(v[i] - (double)(float)v[i]));
    } else {
      for (size_t i = 0; i < len; ++i) out.push_back(v[i]);
    }
    while (out.size() % 4) out.push_back(0.0);
  }
  pt.offset = off;
  return out;
}

int choose_split(int64_t N, std::vector<int>& rs, int64_t single_max, int prec, bool may_reorder) {
  // pass grouping: one group when a transform fits one CTA's shared memory, else split the
  // sequence after the prefix whose product P best balances P against N/P
  const int64_t single = single_max > 0 ? std::min(single_max, max_single_group(prec))
                                        : max_single_group(prec);
  int split = split_point(N, rs, single);
  // no split within the preferred group size: allow groups up to the shared-memory limit, and
  // (for a planner-chosen order) reorder the radices around the most balanced factor pair
  if (split < 0) split = split_point(N, rs, max_single_group(prec));
  if (split < 0 && may_reorder) {
    std::vector<int> bal = balanced_radices(N);
    const int s2 = bal.empty() ? -1 : split_point(N, bal, max_single_group(prec));
    if (s2 >= 0) {
      rs = bal;
      split = s2;
    }
  }
  return split;
}

std::string build_c2c(Plan& p, int64_t tile_target) {
  const int64_t N = p.n;
  const int prec = p.precision;
  std::vector<int>& rs = p.radices;
  std::string msg = check_radices(N, rs);
  if (!msg.empty()) return msg;
  const int split = choose_split(N, rs, p.single_max, prec, !p.radices_given);
  if (split < 0) return "size too large for two pass groups with this radix order";
  PassTables pt = make_pass_tables(N, p.fwd, rs, prec);
  const std::vector<int> comp = compensated_passes(N, rs, split, p.no_comp ? 0 : prec);
  if (prec == 1) pt.values = split_compensated(pt, rs, comp);
  // binary32 two-group plans over contiguous lines whose two groups both have a
  // register-staged kernel: the second group reads its tables in pass order
  p.direct_variant[0] = p.direct_variant[1] = -1;
  if (prec == 1 && split > 0 && split < (int)rs.size() && !p.generic_kernels &&
      p.howmany2 == 1 && p.in.stride == 1 && p.out.stride == 1 && direct_enabled()) {
    int64_t P = 1;
    for (int t = 0; t < split; ++t) P *= rs[t];
    const int v1 = direct_variant_f32(kDirectFirstOfTwo, (int)P, (int)(N / P), false, rs.data(),
                                      split);
    const int v2 = direct_variant_f32(kDirectSecondOfTwo, (int)(N / P), (int)P, comp[split] != 0,
                                      rs.data() + split, (int)rs.size() - split);
    if (v1 >= 0 && v2 >= 0) {
      p.direct_variant[0] = v1;
      p.direct_variant[1] = v2;
    }
  }
  if (p.direct_variant[1] < 0) transpose_second_group(pt, rs, split, comp);
  // the register-staged kernels read a compensated twiddle as one (hi, lo) quadruple
  interleave_tables(pt, rs, comp, p.direct_variant[1] >= 0);
  p.d_twiddles = upload_tables(pt.values, prec, &msg);
  if (!p.d_twiddles) return msg;

  p.flops = plan_ops(N, rs) * (double)p.howmany;
  if (split == (int)rs.size()) {
    p.ngroups = 1;
    GroupDesc& g = p.groups[0];
    fill_group(g, rs, pt, 0, (int)rs.size(), 1, tile_target, prec, p.d_twiddles);
    // lines may share a tile; pick C by the target only (the batch need not divide)
    int64_t cmax = std::max<int64_t>(1, tile_target / N);
    while (cmax > 1 && smem_bytes(cmax, N, prec) > kSmemBudget) --cmax;
    const int64_t lines = p.howmany * p.howmany2;
    g.C = (int)std::min<int64_t>(cmax, std::max<int64_t>(1, lines));
    g.total_sub = lines;
    g.in_elem = p.in.stride;
    g.out_elem = p.out.stride;
    if (p.howmany2 == 1) {
      g.in_line = p.in.dist;
      g.in_sub = 0;
      g.out_line = p.out.dist;
      g.out_sub = 0;
    } else {
      // two batch dimensions: the inner one indexes sub-problems within an outer "line"
      // (a single group's twiddles do not depend on the sub-problem index)
      g.nsub = (int)p.howmany;
      g.in_sub = p.in.dist;
      g.out_sub = p.out.dist;
      g.in_line = p.in_dist2;
      g.out_line = p.out_dist2;
    }
    p.group_first_pass[0] = 0;
  } else {
    p.ngroups = 2;
    int64_t P = 1;
    for (int t = 0; t < split; ++t) P *= rs[t];
    const int64_t Q = N / P;
    GroupDesc& g1 = p.groups[0];
    GroupDesc& g2 = p.groups[1];
    fill_group(g1, rs, pt, 0, split, Q, tile_target, prec, p.d_twiddles);
    fill_group(g2, rs, pt, split, (int)rs.size(), P, tile_target, prec, p.d_twiddles);
    g1.total_sub = p.howmany * Q;
    g2.total_sub = p.howmany * P;
    // group 1: sub-problem b reads x[b + Q*i], writes z[b*P + m]; the intermediate z
    // layout (line, stride) is filled in at execution (out, or the scratch buffer)
    g1.in_line = p.in.dist;
    g1.in_sub = p.in.stride;
    g1.in_elem = Q * p.in.stride;
    // group 2: sub-problem m reads z[i*P + m] and writes out[o*P + m]
    g2.out_line = p.out.dist;
    g2.out_sub = p.out.stride;
    g2.out_elem = P * p.out.stride;
    p.group_first_pass[0] = 0;
    p.group_first_pass[1] = split;
  }
  for (int gi = 0; gi < p.ngroups; ++gi)
    for (int t = 0; t < p.groups[gi].npass; ++t)
      p.groups[gi].pass[t].comp = comp[p.group_first_pass[gi] + t];
  // a lone binary64 transform of a contiguous line: the thread-block cluster kernel
  p.cluster = false;
  if (p.d_cluster_img) cudaFree(p.d_cluster_img);
  p.d_cluster_img = nullptr;
  if (prec == 0 && p.ngroups == 1 && p.howmany == 1 && p.howmany2 == 1 && p.stages.empty() &&
      p.in.stride == 1 && p.out.stride == 1 && cluster_size_f64(p.groups[0]) > 0) {
    std::vector<unsigned char> img;
    ClusterArgs ca{};
    if (build_cluster_image_f64(p.groups[0], p.fwd, pt.values.data(), pt.offset.data(), img, &ca) > 0 &&
        cluster_smem_bytes_f64(ca) <= kSmemBudget &&
        cudaMalloc(&p.d_cluster_img, img.size()) == cudaSuccess) {
      if (cudaMemcpy(p.d_cluster_img, img.data(), img.size(), cudaMemcpyHostToDevice) == cudaSuccess) {
        ca.img = p.d_cluster_img;
        p.cluster_args = ca;
        p.cluster = true;
      } else {
        cudaFree(p.d_cluster_img);
        p.d_cluster_img = nullptr;
      }
    }
  }
  // binary32 over back-to-back lines: the persistent kernel with bulk-copy prefetch
  const GroupDesc& g0 = p.groups[0];
  if (prec == 1 && p.ngroups == 1 && p.howmany2 == 1 && p.in.stride == 1 && p.out.stride == 1 &&
      p.in.dist == N &&
      p.out.dist == N && (N % 2) == 0 && p.howmany > 0 &&
      smem_bytes(g0.C, g0.M, prec) * 2 <= kSmemBudget) {
    if (cudaMalloc(&p.d_status, sizeof(int)) == cudaSuccess &&
        cudaMemset(p.d_status, 0, sizeof(int)) == cudaSuccess) {
      int dev = 0, sms = 1;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      const int64_t tiles = (p.howmany + g0.C - 1) / g0.C;
      bool any_comp = false;
      for (int t = 0; t < g0.npass; ++t) any_comp = any_comp || g0.pass[t].comp;
      p.stream_variant = any_comp || p.generic_kernels ? -1 : stream_variant_f32(N, rs);
      const int64_t want = (int64_t)sms * stream_blocks_per_sm_f32(g0, p.stream_variant);
      p.stream_grid = (unsigned)std::max<int64_t>(1, std::min(want, tiles));
      p.stream = true;
    }
  }
  // binary32 one-group plans of 2^9 .. 2^12 points over contiguous lines: the register-staged
  // kernel (the bulk-copy kernel stays for the bounded-wait tests, which need its waits)
  if (prec == 1 && p.ngroups == 1 && p.howmany2 == 1 && p.in.stride == 1 && p.out.stride == 1 &&
      p.howmany > 0 && !p.generic_kernels && !p.wait_give_up && direct_enabled()) {
    bool any_comp = false;
    for (int t = 0; t < g0.npass; ++t) any_comp = any_comp || g0.pass[t].comp;
    if (!any_comp)
      p.direct_variant[0] = direct_variant_f32(kDirectSingle, (int)N, 1, false, rs.data(),
                                               (int)rs.size());
  }
  // one-butterfly sizes (N <= 16, one untwiddled pass): the warp-tile kernel, ahead of the
  // group and bulk-copy kernels
  p.small_grid = 0;
  if (p.ngroups == 1 && p.howmany2 == 1 && p.stages.empty() && p.howmany > 0 && !p.cluster &&
      !p.generic_kernels && !p.wait_give_up && small_enabled() && small_kernel_applies(g0, prec) &&
      small_preferred(prec, N, g0.npass, p.stream) && prepare_small_kernels() == cudaSuccess)
    p.small_grid = small_grid(g0, prec);
  if (prec == 1 && !p.stream && p.howmany > 0) {
    // three tile buffers per CTA (stage + two work buffers): shrink C to fit
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    bool fits = true;
    for (int gi = 0; gi < p.ngroups; ++gi) {
      GroupDesc& g = p.groups[gi];
      while (g.C > 1 && smem_bytes(g.C, g.M, prec) / 2 * 3 > kSmemBudget) --g.C;
      if (smem_bytes(g.C, g.M, prec) / 2 * 3 > kSmemBudget) fits = false;
    }
    if (fits) {
      for (int gi = 0; gi < p.ngroups; ++gi) {
        GroupDesc& g = p.groups[gi];
        set_divisors(g);
        int v = p.ngroups == 2 && !p.generic_kernels ? tile_variant_f32(g) : -1;
        if (v >= 0 && tile_stream_smem_bytes_f32(g, v) > kSmemBudget) v = -1;
        p.ts_variant[gi] = v;
        const int64_t tiles = (g.total_sub + g.C - 1) / g.C;
        const int64_t want = (int64_t)sms * tile_stream_blocks_per_sm_f32(g, v);
        p.ts_grid[gi] = (unsigned)std::max<int64_t>(1, std::min(want, tiles));
      }
      p.tile_stream = true;
    }
  }
  return "";
}

std::string build_real(Plan& p, const RealLayout& L, int64_t tile_target) {
  const int prec = p.precision;
  const bool r2c = p.kind == Kind::R2C;
  const int64_t N = L.n, M = N / 2;
  if (N < 2 || (N & 1)) return "real transforms of odd size are not executed on the GPU";
  if ((L.r_off & 1) || (L.r_bdist & 1) || (L.r_rdist & 1))
    return "real lines must start at even double offsets";
  const int64_t max_m = max_single_group(prec);
  if (M > max_m) return "real transform too large for one pass group";
  p.n = N;
  RealDesc& d = p.real;
  d.M = (int)M;
  d.rows = L.n0;
  d.lines = L.howmany * L.n0;
  d.r_off = L.r_off;
  d.r_bdist = L.r_bdist;
  d.r_rdist = L.r_rdist;
  d.c_off = L.c_off;
  d.c_bdist = L.c_bdist;
  d.c_rdist = L.c_rdist;
  std::string msg;
  // size-M passes (none for M = 1)
  p.radices = M >= 2 ? choose_radices(M, prec) : std::vector<int>{};
  PassTables pt;
  if (M >= 2) {
    msg = check_radices(M, p.radices);
    if (!msg.empty()) return msg;
    pt = make_pass_tables(M, r2c, p.radices, prec);
    interleave_tables(pt, p.radices, {});
  }
  p.d_twiddles = upload_tables(pt.values, prec, &msg);
  if (!p.d_twiddles) return msg;
  if (M >= 2) {
    fill_group(d.g, p.radices, pt, 0, (int)p.radices.size(), 1, tile_target, prec, p.d_twiddles);
  } else {
    d.g.M = 1;
    d.g.npass = 0;
    d.g.nsub = 1;
    d.g.scale = 1.0;
  }
  int64_t cmax = std::max<int64_t>(1, tile_target / std::max<int64_t>(M, 1));
  while (cmax > 1 && smem_bytes(cmax, M, prec) > kSmemBudget) --cmax;
  d.g.C = (int)std::min<int64_t>(cmax, std::max<int64_t>(1, d.lines));
  // binary32 r2c rows of a power-of-two size with a register-staged kernel
  d.direct = prec == 1 && r2c && !p.generic_kernels && M >= 2
                 ? r2c_rows_variant_f32((int)M, p.radices.data(), (int)p.radices.size())
                 : -1;
  // split twiddles cos/sin(2 pi k / N), k = 0..M/2, halved for r2c
  std::vector<double> tab = cos_sin_2pi_table((uint64_t)N);
  // [halved table | full table]
  const int64_t np = M / 2 + 1;
  std::vector<double> post(4 * np);
  for (int64_t k = 0; k < np; ++k) {
    post[2 * k] = r2c ? 0.5 * tab[2 * k] : tab[2 * k];
    post[2 * k + 1] = r2c ? 0.5 * tab[2 * k + 1] : tab[2 * k + 1];
    post[2 * np + 2 * k] = tab[2 * k];
    post[2 * np + 2 * k + 1] = tab[2 * k + 1];
  }
  p.d_post = upload_tables(post, prec, &msg);
  if (!p.d_post) return msg;
  d.post = p.d_post;
  d.post_full = prec == 0 ? (const void*)((const double*)p.d_post + 2 * np)
                          : (const void*)((const float*)p.d_post + 2 * np);
  p.flops = (plan_ops(M, p.radices) + 6.0 * M) * (double)d.lines;
  // rank 2: complex transform of length n0 along the first axis of the half spectrum
  p.has_col = L.n0 > 1;
  if (p.has_col) {
    std::vector<int> crs = choose_radices(L.n0, prec);
    msg = check_radices(L.n0, crs);
    if (!msg.empty()) return msg;
    if (L.n0 > max_m) return "first dimension too large for one pass group";
    PassTables ct = make_pass_tables(L.n0, r2c, crs, prec);
    interleave_tables(ct, crs, {});
    p.d_col_twiddles = upload_tables(ct.values, prec, &msg);
    if (!p.d_col_twiddles) return msg;
    const int64_t h = M + 1;
    GroupDesc& g = p.col;
    fill_group(g, crs, ct, 0, (int)crs.size(), 1, tile_target, prec, p.d_col_twiddles);
    int64_t cm = std::max<int64_t>(1, tile_target / L.n0);
    // columns are copied as runs of C neighbouring elements: keep binary32 runs at 64 bytes
    if (prec == 1) cm = std::max<int64_t>(cm, 8);
    while (cm > 1 && smem_bytes(cm, L.n0, prec) > kSmemBudget) --cm;
    // columns of one image are the sub-problems; tiles may straddle images (no sub-problem
    // index enters the twiddles of a single group)
    g.nsub = (int)h;
    g.total_sub = L.howmany * h;
    g.C = (int)std::min<int64_t>(cm, g.total_sub);
    g.in_sub = g.out_sub = 1;
    if (r2c) {   // in place on the output
      g.in_line = g.out_line = L.c_bdist;
      g.in_elem = g.out_elem = L.c_rdist;
    } else {     // from the input to a contiguous scratch image, then rows from the scratch
      g.in_line = L.c_bdist;
      g.in_elem = L.c_rdist;
      g.out_line = L.n0 * h;
      g.out_elem = h;
      p.col_in_off = L.c_off;
      d.c_off = 0;
      // the column transform's output, allocated with the plan
      const size_t need = (size_t)L.howmany * L.n0 * h * (prec == 0 ? 16 : 8);
      if (cudaMalloc(&p.d_scratch, need) != cudaSuccess) return "cudaMalloc of the c2r scratch failed";
      p.scratch_bytes = need;
      d.c_bdist = L.n0 * h;
      d.c_rdist = h;
    }
    p.flops += plan_ops(L.n0, crs) * (double)(L.howmany * h);
    // binary32 columns of a power-of-two length: the register-staged column kernel
    p.col_direct = prec == 1 && !p.generic_kernels
                       ? direct_cols_variant_f32((int)L.n0, crs.data(), (int)crs.size())
                       : -1;
    // binary32 columns: the persistent strided-tile kernel (the next tile's elements copied
    // asynchronously under the current tile's passes) when its three tile buffers fit
    if (prec == 1 && smem_bytes(g.C, g.M, prec) / 2 * 3 <= kSmemBudget) {
      int dev = 0, sms = 1;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      GroupDesc gs = g;
      set_divisors(gs);
      const int64_t tiles = (g.total_sub + g.C - 1) / g.C;
      const int64_t want = (int64_t)sms * tile_stream_blocks_per_sm_f32(gs);
      p.col_ts_grid = (unsigned)std::max<int64_t>(1, std::min(want, tiles));
    }
  }
  return "";
}

// The intermediate buffer of in-place two-group execution (one block of lines), allocated on
// first use and kept by the plan.
static cudaError_t ensure_scratch_bytes(const Plan& p, size_t need) {
  if (p.scratch_bytes >= need) return cudaSuccess;
  if (p.d_scratch) cudaFree(p.d_scratch);
  p.d_scratch = nullptr;
  p.scratch_bytes = 0;
  cudaError_t e = cudaMalloc(&p.d_scratch, need);
  if (e == cudaSuccess) p.scratch_bytes = need;
  return e;
}

static cudaError_t ensure_scratch(const Plan& p) {
  return ensure_scratch_bytes(p, (size_t)p.n * (size_t)p.howmany * (p.precision == 0 ? 16 : 8));
}

cudaError_t execute_plan(const Plan& p, const void* in, void* out, cudaStream_t stream,
                         bool force_scratch, void* scratch) {
  if (p.empty) return cudaSuccess;
  if (p.generic) {
    const size_t ces = p.precision == 0 ? 16 : 8;
    return launch_generic(p.gen, p.precision, p.fwd, static_cast<const char*>(in) + p.in.offset * (int64_t)ces,
                          static_cast<char*>(out) + p.out.offset * (int64_t)ces, stream);
  }
  if (!p.steps.empty()) {
    const size_t ces = p.precision == 0 ? 16 : 8;
    void* bufs[4] = {const_cast<void*>(in), out, p.d_pack_buf,
                     static_cast<char*>(p.d_pack_buf) + (size_t)p.pack_elems * ces};
    for (const PackStep& st : p.steps) {
      cudaError_t e;
      if (st.op == PackStep::kGather) e = launch_pack(st.pd, p.precision, bufs[st.src], bufs[st.dst], stream);
      else if (st.op == PackStep::kScatter) e = launch_unpack(st.pd, p.precision, bufs[st.src], bufs[st.dst], stream);
      else e = execute_plan(*st.plan, bufs[st.src], bufs[st.dst], stream);
      if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
  }
  if (p.chirp_fwd) {
    // Bluestein: chirp and pad -> forward L -> filter -> backward L (scaled 1/L) -> chirp
    const size_t ces = p.precision == 0 ? 16 : 8;
    char* A = static_cast<char*>(p.d_chirp_buf);
    char* B = A + (size_t)p.chirp.lines * (size_t)p.chirp.L * ces;
    const char* ib = static_cast<const char*>(in) + p.in.offset * (int64_t)ces;
    char* ob = static_cast<char*>(out) + p.out.offset * (int64_t)ces;
    cudaError_t e = launch_chirp_pre(p.chirp, p.precision, ib, A, stream);
    if (e == cudaSuccess) e = execute_plan(*p.chirp_fwd, A, B, stream);
    if (e == cudaSuccess) e = launch_chirp_mul(p.chirp, p.precision, B, stream);
    if (e == cudaSuccess) e = execute_plan(*p.chirp_bwd, B, A, stream);
    if (e == cudaSuccess) e = launch_chirp_post(p.chirp, p.precision, A, ob, stream);
    return e;
  }
  if (p.kind == Kind::R2R && p.stages.empty()) {
    // embedding -> complex DFT of the embedding size -> extraction
    const size_t ces = p.precision == 0 ? 16 : 8;
    char* A = static_cast<char*>(p.d_r2r_buf);
    char* B = A + (size_t)p.r2r.lines * (size_t)p.r2r.M * ces;
    cudaError_t e = launch_r2r_embed(p.r2r, p.precision, in, A, stream);
    if (e != cudaSuccess) return e;
    if (p.r2r_dft) {
      e = execute_plan(*p.r2r_dft, A, B, stream);
      if (e != cudaSuccess) return e;
    } else {
      B = A;
    }
    return launch_r2r_extract(p.r2r, p.precision, B, out, stream);
  }
  if (!p.stages.empty()) {
    // axis by axis: the first stage reads the input, the others work in place on the output
    const size_t es = p.kind == Kind::R2R ? (p.precision == 0 ? 8 : 4) : (p.precision == 0 ? 16 : 8);
    for (size_t k = 0; k < p.stages.size(); ++k) {
      const AxisStage& st = p.stages[k];
      const char* src = k == 0 ? static_cast<const char*>(in) : static_cast<const char*>(out);
      for (const auto& off : st.loops) {
        cudaError_t e = execute_plan(*st.plan, src + off[0] * (int64_t)es,
                                     static_cast<char*>(out) + off[1] * (int64_t)es, stream,
                                     force_scratch);
        if (e != cudaSuccess) return e;
      }
    }
    return cudaSuccess;
  }
  if (p.howmany2 > 1 && p.ngroups == 2) {
    // two pass groups use the sub-problem index themselves: one launch pair per outer block,
    // sharing the plan's scratch (allocated here, so the blocks never reallocate it)
    const size_t es = p.precision == 0 ? 16 : 8;
    cudaError_t e = (in == out || force_scratch) ? ensure_scratch(p) : cudaSuccess;
    if (e != cudaSuccess) return e;
    Plan q = p;
    q.howmany2 = 1;
    q.stages.clear();
    for (int64_t j = 0; j < p.howmany2 && e == cudaSuccess; ++j)
      e = execute_plan(q, static_cast<const char*>(in) + j * p.in_dist2 * (int64_t)es,
                       static_cast<char*>(out) + j * p.out_dist2 * (int64_t)es, stream,
                       force_scratch);
    return e;
  }
  const size_t es = p.precision == 0 ? 16 : 8;
  auto launch_col = [&](bool fwd, const void* a, void* b) -> cudaError_t {
    if (p.precision == 0) return launch_group_f64(p.col, fwd, a, b, stream);
    if (p.col_direct >= 0) return launch_direct_cols_f32(p.col, fwd, a, b, p.col_direct, stream);
    if (p.col_ts_grid && ((uintptr_t)a % 8) == 0 && ((uintptr_t)b % 8) == 0)
      return launch_tile_stream_f32(p.col, fwd, a, b, p.col_ts_grid, stream);
    return launch_group_f32(p.col, fwd, a, b, stream);
  };
  if (p.kind == Kind::R2C) {
    if (force_scratch && p.has_col) {
      // host-mapped buffers: the rows go to a device copy of the output span and the column
      // pass reads them there, so the half spectrum crosses the host link once
      cudaError_t e = ensure_scratch_bytes(p, (size_t)p.out_span * (p.precision == 0 ? 8 : 4));
      if (e != cudaSuccess) return e;
      if ((e = launch_real(p.real, p.precision, true, in, p.d_scratch, stream)) != cudaSuccess) return e;
      const int64_t off = p.real.c_off * (int64_t)es;
      return launch_col(true, static_cast<char*>(p.d_scratch) + off, static_cast<char*>(out) + off);
    }
    cudaError_t e = launch_real(p.real, p.precision, true, in, out, stream);
    if (e != cudaSuccess || !p.has_col) return e;
    char* ob = static_cast<char*>(out) + p.real.c_off * (int64_t)es;
    return launch_col(true, ob, ob);
  }
  if (p.kind == Kind::C2R) {
    if (!p.has_col) return launch_real(p.real, p.precision, false, in, out, stream);
    const char* ib = static_cast<const char*>(in) + p.col_in_off * (int64_t)es;
    cudaError_t e = launch_col(false, ib, p.d_scratch);
    if (e != cudaSuccess) return e;
    return launch_real(p.real, p.precision, false, p.d_scratch, out, stream);
  }
  const char* ib = static_cast<const char*>(in) + p.in.offset * (int64_t)es;
  char* ob = static_cast<char*>(out) + p.out.offset * (int64_t)es;
  auto launch = [&](int gi, const GroupDesc& g, const void* a, void* b) -> cudaError_t {
    if (p.precision == 0) return launch_group_f64(g, p.fwd, a, b, stream);
    // (its tables are laid out for it: no other kernel may run this group)
    if (p.direct_variant[gi] >= 0) return launch_direct_f32(g, p.fwd, a, b, p.direct_variant[gi], stream);
    if (p.tile_stream && ((uintptr_t)a % 8) == 0 && ((uintptr_t)b % 8) == 0)
      return launch_tile_stream_f32(g, p.fwd, a, b, p.ts_grid[gi], stream, p.ts_variant[gi]);
    return launch_group_f32(g, p.fwd, a, b, stream);
  };
  if (p.ngroups == 1) {
    if (p.direct_variant[0] >= 0)
      return launch_direct_f32(p.groups[0], p.fwd, ib, ob, p.direct_variant[0], stream);
    if (p.cluster && ((uintptr_t)ib % 16) == 0 && ((uintptr_t)ob % 16) == 0)
      return launch_cluster_f64(p.cluster_args, p.groups[0].scale, ib, ob, stream);
    if (p.small_grid)
      return launch_small(p.groups[0], p.precision, p.fwd, ib, ob, p.small_grid, stream);
    // the bulk-copy engine needs 16-byte aligned ranges; in place is fine (each tile is read
    // into shared memory before it is written)
    if (p.stream && ((uintptr_t)ib % 16) == 0 && ((uintptr_t)ob % 16) == 0)
      return launch_stream_f32(p.groups[0], p.fwd, ib, ob, p.howmany, p.stream_grid, p.d_status,
                               stream, p.wait_give_up, p.stream_variant);
    return launch(0, p.groups[0], ib, ob);
  }
  // two groups: the intermediate goes to `out` when it does not alias the input, else to the
  // plan's scratch buffer (allocated on first use)
  GroupDesc g1 = p.groups[0], g2 = p.groups[1];
  const int64_t P = g2.nsub;
  char* zb;
  int64_t z_line, z_stride;
  if (in != out && !force_scratch) {
    zb = ob;
    z_line = p.out.dist;
    z_stride = p.out.stride;
  } else {
    if (!scratch) {
      cudaError_t e = ensure_scratch(p);
      if (e != cudaSuccess) return e;
    }
    zb = static_cast<char*>(scratch ? scratch : p.d_scratch);
    z_line = p.n;
    z_stride = 1;
  }
  g1.out_line = z_line;
  g1.out_sub = P * z_stride;
  g1.out_elem = z_stride;
  g2.in_line = z_line;
  g2.in_sub = z_stride;
  g2.in_elem = P * z_stride;
  cudaError_t e = launch(0, g1, ib, zb);
  if (e != cudaSuccess) return e;
  return launch(1, g2, zb, ob);
}

}  // namespace lfg
