// Device autotuner (LFG_MEASURE): lean-fftw's measuring planner restated for the GPU.
//
// lean-fftw enumerates radix sequences ("a first radix, then a monotone tail",
// LeanFFTW/Asm/Planner.lean:40-94), prunes candidates whose proved operation count exceeds the
// best by 1.5x (`raceOrder`, :193-205), times the rest on the CPU and re-times the leaders
// (:270-286).  Here the candidates are (radix sequence, pass grouping, tile size); sequences
// come from the same enumeration pruned at 1.15x of the fewest codelet operations (on GB300
// the binary64 path is bound by the FP64 pipe, so operation count is nearly the whole cost);
// each candidate is timed with CUDA events on scratch buffers of the plan's own shape, and
// the fastest is kept.  With LFG_PLAN_LOG set, every measured candidate is appended to that
// file as one JSON line (the analogue of LF_PLAN_LOG, Planner.lean:162-168).
//
// Tuning cache ("wisdom"; lean-fftw has none and re-measures every plan): every choice the
// autotuner makes is remembered in a process-wide table keyed by the problem (size,
// precision, direction and scratch batch for a 1-D plan; a hash of the sizes and offsets for
// a ragged batch), and a later LFG_MEASURE plan of the same problem takes the stored choice
// without timing anything.  The table is read from and appended to the file named by
// LFG_WISDOM, and lfg_wisdom_import/export/forget move it explicitly.  One entry per line:
// `key<TAB>value`; lines starting with '#' are comments.  An entry that does not describe a
// valid schedule for its problem is ignored and the problem is measured again.
#include "tuner.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <map>
#include <mutex>
#include <sstream>

#include "generated/opcounts.h"
#include "kernels.h"
#include "ragged.h"

namespace lfg {

std::vector<std::vector<int>> candidate_radices(int64_t n, double slack, size_t max_count) {
  std::vector<std::pair<double, std::vector<int>>> all;
  std::vector<int> cur;
  // first radix R0 (untwiddled), then a non-increasing tail of twiddled radices
  std::function<void(int64_t, int, double)> tail = [&](int64_t m, int maxr, double cost) {
    if (m == 1) {
      all.push_back({cost, cur});
      return;
    }
    if ((int)cur.size() >= kMaxPass || all.size() > 20000) return;
    for (int R = std::min<int64_t>(maxr, m); R >= 2; --R) {
      if (m % R || !radix_ok(R)) continue;
      cur.push_back(R);
      tail(m / R, R, cost + (double)kOpsTw[R] / R);
      cur.pop_back();
    }
  };
  for (int R0 = kMaxRadix; R0 >= 2; --R0) {
    if (n % R0 || !radix_ok(R0)) continue;
    cur.assign(1, R0);
    tail(n / R0, kMaxRadix, (double)kOpsUntw[R0] / R0);
  }
  std::sort(all.begin(), all.end(), [](const auto& a, const auto& b) {
    return a.first < b.first || (a.first == b.first && a.second.size() < b.second.size());
  });
  std::vector<std::vector<int>> out;
  if (all.empty()) return out;
  const double best = all.front().first;
  for (auto& c : all) {
    if (c.first > best * slack || out.size() >= max_count) break;
    out.push_back(c.second);
  }
  return out;
}

namespace {

void log_line(const std::string& s) {
  const char* path = std::getenv("LFG_PLAN_LOG");
  if (!path || !*path) return;
  if (FILE* f = std::fopen(path, "a")) {
    std::fputs(s.c_str(), f);
    std::fputc('\n', f);
    std::fclose(f);
  }
}

std::string seq_str(const std::vector<int>& rs) {
  std::string s = "[";
  for (size_t i = 0; i < rs.size(); ++i) s += (i ? "," : "") + std::to_string(rs[i]);
  return s + "]";
}

// Median of `reps` timed executions (after one warm-up) of fn on a private stream.
template <class F>
float time_ms(F fn, cudaStream_t s, int reps) {
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  fn(s);
  std::vector<float> t;
  for (int i = 0; i < reps; ++i) {
    cudaEventRecord(a, s);
    fn(s);
    cudaEventRecord(b, s);
    cudaEventSynchronize(b);
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    t.push_back(ms);
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  std::sort(t.begin(), t.end());
  return t.empty() ? INFINITY : t[t.size() / 2];
}


// ---- tuning cache ---------------------------------------------------------------------------
std::mutex g_wisdom_mu;
std::map<std::string, std::string> g_wisdom;
bool g_wisdom_env_read = false;

bool read_wisdom_locked(const char* path) {
  FILE* f = std::fopen(path, "r");
  if (!f) return false;
  char buf[8192];
  while (std::fgets(buf, sizeof buf, f)) {
    std::string line(buf);
    while (!line.empty() && (line.back() == '\n' || line.back() == '\r')) line.pop_back();
    if (line.empty() || line[0] == '#') continue;
    const size_t tab = line.find('\t');
    if (tab == std::string::npos || tab == 0 || tab + 1 >= line.size()) continue;
    g_wisdom[line.substr(0, tab)] = line.substr(tab + 1);
  }
  std::fclose(f);
  return true;
}

const char* wisdom_env() {
  const char* p = std::getenv("LFG_WISDOM");
  return p && *p ? p : nullptr;
}

void read_env_wisdom_locked() {
  if (g_wisdom_env_read) return;
  g_wisdom_env_read = true;
  if (const char* p = wisdom_env()) read_wisdom_locked(p);
}

bool recall(const std::string& key, std::string* value) {
  std::lock_guard<std::mutex> lk(g_wisdom_mu);
  read_env_wisdom_locked();
  auto it = g_wisdom.find(key);
  if (it == g_wisdom.end()) return false;
  *value = it->second;
  return true;
}

void remember(const std::string& key, const std::string& value) {
  std::lock_guard<std::mutex> lk(g_wisdom_mu);
  read_env_wisdom_locked();
  g_wisdom[key] = value;
  if (const char* p = wisdom_env())
    if (FILE* f = std::fopen(p, "a")) {
      std::fprintf(f, "%s\t%s\n", key.c_str(), value.c_str());
      std::fclose(f);
    }
}

// value fields "name=v1,v2,...;name=..." -> integers of one field (empty if absent or malformed)
std::vector<int64_t> field(const std::string& value, const char* name) {
  std::vector<int64_t> out;
  const std::string tag = std::string(name) + "=";
  size_t pos = 0;
  while (pos < value.size()) {
    size_t end = value.find(';', pos);
    if (end == std::string::npos) end = value.size();
    if (value.compare(pos, tag.size(), tag) == 0) {
      std::stringstream ss(value.substr(pos + tag.size(), end - pos - tag.size()));
      std::string tok;
      while (std::getline(ss, tok, ',')) {
        char* e = nullptr;
        const long long v = std::strtoll(tok.c_str(), &e, 10);
        if (tok.empty() || *e) return {};
        out.push_back(v);
      }
      return out;
    }
    pos = end + 1;
  }
  return out;
}

uint64_t fnv1a(uint64_t h, const void* p, size_t bytes) {
  const unsigned char* c = static_cast<const unsigned char*>(p);
  for (size_t i = 0; i < bytes; ++i) h = (h ^ c[i]) * 1099511628211ull;
  return h;
}

}  // namespace

bool wisdom_import(const char* path) {
  std::lock_guard<std::mutex> lk(g_wisdom_mu);
  read_env_wisdom_locked();
  return read_wisdom_locked(path);
}

bool wisdom_export(const char* path) {
  std::lock_guard<std::mutex> lk(g_wisdom_mu);
  read_env_wisdom_locked();
  FILE* f = std::fopen(path, "w");
  if (!f) return false;
  std::fprintf(f, "# lean-fftw GB300 tuning cache: key<TAB>value\n");
  for (const auto& kv : g_wisdom) std::fprintf(f, "%s\t%s\n", kv.first.c_str(), kv.second.c_str());
  return std::fclose(f) == 0;
}

void wisdom_forget() {
  std::lock_guard<std::mutex> lk(g_wisdom_mu);
  g_wisdom.clear();
  g_wisdom_env_read = true;   // a forgotten table is not re-read from LFG_WISDOM
}

size_t wisdom_size() {
  std::lock_guard<std::mutex> lk(g_wisdom_mu);
  read_env_wisdom_locked();
  return g_wisdom.size();
}

std::string tune_c2c(Plan& p, int64_t default_tile) {
  const int prec = p.precision;
  const size_t es = prec == 0 ? 16 : 8;
  // a scratch batch of the plan's line shape, 32-256 MB, contiguous
  const int64_t per_line = p.n;
  int64_t lines = std::max<int64_t>(1, std::min<int64_t>(p.howmany, ((int64_t)256 << 20) / (per_line * es)));
  lines = std::max<int64_t>(lines, std::min<int64_t>(p.howmany, ((int64_t)32 << 20) / (per_line * es)));
  const std::string key = "c2c n=" + std::to_string(p.n) + " precision=" + std::to_string(prec) +
                          " fwd=" + std::to_string(p.fwd ? 1 : 0) + " lines=" + std::to_string(lines);
  {
    std::string v;
    if (recall(key, &v)) {
      const std::vector<int64_t> rs = field(v, "radices"), sm = field(v, "single"), tl = field(v, "tile");
      std::vector<int> r(rs.begin(), rs.end());
      if (!rs.empty() && sm.size() == 1 && tl.size() == 1 && check_radices(p.n, r).empty() &&
          sm[0] >= 2 && tl[0] >= 16 && tl[0] <= 65536) {
        p.radices = r;
        p.single_max = sm[0];
        p.tile = tl[0];
        return "";
      }
    }
  }
  void *din = nullptr, *dout = nullptr;
  const size_t bytes = (size_t)lines * per_line * es;
  if (cudaMalloc(&din, bytes) != cudaSuccess) return "autotuner: scratch allocation failed";
  if (cudaMalloc(&dout, bytes) != cudaSuccess) {
    cudaFree(din);
    return "autotuner: scratch allocation failed";
  }
  cudaMemset(din, 0x3F, bytes);   // finite, normal binary64 / binary32 values
  cudaStream_t s;
  cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);

  std::vector<std::vector<int>> seqs = candidate_radices(p.n, 1.15, 6);
  if (prec == 1) {   // the balanced binary32 order (choose_radices) is always a candidate
    const std::vector<int> bal = choose_radices(p.n, prec);
    if (std::find(seqs.begin(), seqs.end(), bal) == seqs.end()) seqs.push_back(bal);
  }
  std::vector<int64_t> splits = prec == 0 ? std::vector<int64_t>{1024, 2048, 4096, 1 << 30}
                                          : std::vector<int64_t>{kF32SingleGroupMax, 1 << 30};
  std::vector<int64_t> tiles = {1024, 2048, 4096};
  float best = INFINITY;
  Plan chosen;
  bool have = false;
  int64_t best_tile = default_tile;
  for (const auto& rs : seqs) {
    std::vector<int> seen_splits;
    for (int64_t sm : splits) {
      const int split = split_point(p.n, rs, std::min<int64_t>(sm, max_single_group(prec)));
      if (split < 0 || std::find(seen_splits.begin(), seen_splits.end(), split) != seen_splits.end())
        continue;
      seen_splits.push_back(split);
      for (int64_t tile : tiles) {
        Plan c = p;
        c.howmany = lines;
        c.in = Side{0, 1, p.n};
        c.out = Side{0, 1, p.n};
        c.radices = rs;
        c.single_max = sm;
        c.d_twiddles = c.d_scratch = c.d_host_in = c.d_host_out = nullptr;
        c.d_cluster_img = nullptr;
        std::string msg = build_c2c(c, tile);
        if (!msg.empty()) {
          free_plan_memory(c);
          continue;
        }
        float ms = time_ms([&](cudaStream_t st) { execute_plan(c, din, dout, st); }, s, 3);
        log_line("{\"n\":" + std::to_string(p.n) + ",\"precision\":" + std::to_string(prec) +
                 ",\"radices\":" + seq_str(rs) + ",\"groups\":" + std::to_string(c.ngroups) +
                 ",\"single_max\":" + std::to_string(sm) + ",\"tile\":" + std::to_string(tile) +
                 ",\"lines\":" + std::to_string(lines) + ",\"ms\":" + std::to_string(ms) + "}");
        free_plan_memory(c);
        if (ms < best) {
          best = ms;
          chosen = p;
          chosen.radices = rs;
          chosen.single_max = sm;
          best_tile = tile;
          have = true;
        }
      }
    }
  }
  cudaStreamDestroy(s);
  cudaFree(din);
  cudaFree(dout);
  if (!have) return "autotuner: no candidate could be built";
  p.radices = chosen.radices;
  p.single_max = chosen.single_max;
  p.tile = best_tile;
  std::string rs;
  for (size_t i = 0; i < p.radices.size(); ++i) rs += (i ? "," : "") + std::to_string(p.radices[i]);
  remember(key, "radices=" + rs + ";single=" + std::to_string(p.single_max) + ";tile=" +
                    std::to_string(p.tile));
  return "";
}

std::string tune_ragged(RaggedPlan& r, RaggedOptions& opt) {
  const size_t es = r.precision == 0 ? 16 : 8;
  uint64_t h = 1469598103934665603ull;
  h = fnv1a(h, r.sizes.data(), r.sizes.size() * sizeof(int64_t));
  h = fnv1a(h, r.in_off.data(), r.in_off.size() * sizeof(int64_t));
  h = fnv1a(h, r.out_off.data(), r.out_off.size() * sizeof(int64_t));
  for (const auto& kv : opt.radices) {
    h = fnv1a(h, &kv.first, sizeof kv.first);
    h = fnv1a(h, kv.second.data(), kv.second.size() * sizeof(int));
  }
  char hex[17];
  std::snprintf(hex, sizeof hex, "%016llx", (unsigned long long)h);
  const std::string key = "ragged precision=" + std::to_string(r.precision) + " fwd=" +
                          std::to_string(r.fwd ? 1 : 0) + " count=" + std::to_string(r.sizes.size()) +
                          " hash=" + hex;
  {
    std::string v;
    if (recall(key, &v)) {
      const std::vector<int64_t> sh = field(v, "shape"), tl = field(v, "tile"), sm = field(v, "single");
      if (sh.size() == 1 && tl.size() == 1 && sm.size() == 1 && sh[0] >= 0 &&
          sh[0] < kRaggedVariants && tl[0] >= 16 && tl[0] <= 65536 && sm[0] >= 2) {
        opt.variant = (int)sh[0];
        opt.tile_target = tl[0];
        opt.single_max = std::min<int64_t>(sm[0], max_single_group(r.precision));
        return "";
      }
    }
  }
  void *in = nullptr, *out = nullptr;
  if (cudaMalloc(&in, (size_t)r.in_span * es) != cudaSuccess) return "autotuner: scratch allocation failed";
  if (cudaMalloc(&out, (size_t)r.out_span * es) != cudaSuccess) {
    cudaFree(in);
    return "autotuner: scratch allocation failed";
  }
  cudaMemset(in, 0x3F, (size_t)r.in_span * es);
  cudaStream_t s;
  cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  struct Cand {
    int variant;
    int64_t tile, single;
  };
  std::vector<Cand> cands;
  for (int v = 0; v < kRaggedVariants; ++v)
    for (int64_t t : {1024, 2048, 4096})
      for (int64_t sm : {1024, 2048, 4096})
        cands.push_back({v, t, sm});
  float best = INFINITY;
  RaggedOptions chosen = opt;
  RaggedOptions shared = opt;
  shared.table_cache = std::make_shared<std::map<std::pair<int64_t, std::vector<int>>, PassTables>>();
  for (const Cand& c : cands) {
    RaggedPlan t;
    t.precision = r.precision;
    t.fwd = r.fwd;
    t.device = r.device;
    t.use_graph = false;
    t.sizes = r.sizes;
    t.in_off = r.in_off;
    t.out_off = r.out_off;
    RaggedOptions o = shared;
    o.variant = c.variant;
    o.tile_target = c.tile;
    o.single_max = std::min<int64_t>(c.single, max_single_group(r.precision));
    std::string msg = build_ragged(t, o);
    if (msg.empty()) {
      float ms = time_ms([&](cudaStream_t st) { execute_ragged(t, in, out, st); }, s, 3);
      log_line("{\"ragged\":" + std::to_string(r.sizes.size()) + ",\"variant\":" +
               std::to_string(c.variant) + ",\"tile\":" + std::to_string(c.tile) +
               ",\"single_max\":" + std::to_string(c.single) + ",\"ms\":" + std::to_string(ms) + "}");
      if (ms < best) {
        best = ms;
        chosen = o;
      }
    }
    free_ragged(t);
  }
  cudaStreamDestroy(s);
  cudaFree(in);
  cudaFree(out);
  if (!std::isfinite(best)) return "autotuner: no ragged candidate could be built";
  opt = chosen;
  opt.table_cache.reset();
  remember(key, "shape=" + std::to_string(opt.variant) + ";tile=" + std::to_string(opt.tile_target) +
                    ";single=" + std::to_string(opt.single_max));
  return "";
}

}  // namespace lfg
