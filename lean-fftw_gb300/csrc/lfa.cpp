// lean-fftw's fast-engine entry points for C callers, on this library's GPU plans.
//
// lean-fftw's libbench2 backend plans a 1-D complex transform with
// `lfa_plan_measure(N, fwd, in, out)` (LeanFFTW/Asm/Planner.lean:293-302, an exported Lean
// function returning the plan's memory, empty when the engine does not cover N) and runs it
// with `lfa_call(record, in, out)` (LeanFFTW/Asm/Kernels.lean:1203-1204; called in
// bench/backends/bench-leanfftw.c:284-288).  The functions here take the same arguments in
// plain C: the plan is an opaque record pointer (NULL when N is not covered, the reference's
// empty plan), `lfg_lfa_call` has lfa_call's signature, and the record is released with
// `lfg_lfa_release` (the reference drops its Lean array with lean_dec).  Status is kept in
// the record, since lfa_call returns nothing.
#include <cstdint>
#include <new>
#include <string>

#include "handles.h"

namespace {

constexpr uint64_t kMagic = 0x6c66612d72656331ull;   // "lfa-rec1"

struct LfaRecord {
  uint64_t magic = kMagic;
  lfg_plan* plan = nullptr;
  bool inplace = false;
  lfg_status last = LFG_OK;
};

const LfaRecord* as_record(const void* r) {
  const LfaRecord* rec = static_cast<const LfaRecord*>(r);
  return rec && rec->magic == kMagic ? rec : nullptr;
}

bool smooth13(size_t n) {
  static const size_t primes[] = {2, 3, 5, 7, 11, 13};
  for (size_t p : primes)
    while (n % p == 0) n /= p;
  return n == 1;
}

}  // namespace

static const void* plan_measure(size_t N, uint8_t fwd, size_t in, size_t out) {
  // the fast engine's domain: 13-smooth sizes 2..2^24 (bench-leanfftw.c:253-268)
  if (N < 2 || N > ((size_t)1 << 24) || !smooth13(N)) {
    lfg::set_last_error("the fast engine covers 13-smooth sizes 2..2^24");
    return nullptr;
  }
  LfaRecord* rec = new (std::nothrow) LfaRecord;
  if (!rec) {
    lfg::set_last_error("host allocation failed");
    return nullptr;
  }
  // measured plan (the autotuner times candidates on device scratch buffers; the caller's
  // arrays are left as they are, which the reference's contract -- contents overwritten --
  // allows)
  const lfg_status s = lfg_plan_1d(N, fwd ? -1 : 1, 1, LFG_F64, LFG_MEASURE, &rec->plan);
  if (s != LFG_OK) {
    delete rec;
    return nullptr;
  }
  rec->inplace = in == out;
  return rec;
}

extern "C" const void* lfg_lfa_plan_measure(size_t N, uint8_t fwd, size_t in, size_t out) {
  try {
    return plan_measure(N, fwd, in, out);
  } catch (...) {   // (host allocation of an error message) never across the C ABI
    return nullptr;
  }
}

extern "C" void lfg_lfa_call(const void* record, const double* in, double* out) {
  const LfaRecord* rec = as_record(record);
  if (!rec) return;   // (the reference's lfa_call has no error path either)
  const_cast<LfaRecord*>(rec)->last = lfg_execute_host(rec->plan, in, out);   // (guarded)
}

extern "C" lfg_status lfg_lfa_status(const void* record) {
  const LfaRecord* rec = as_record(record);
  if (!rec) return LFG_ERR_INVALID;
  return rec->last;
}

extern "C" void lfg_lfa_release(const void* record) {
  LfaRecord* rec = const_cast<LfaRecord*>(as_record(record));
  if (!rec) return;
  lfg_destroy(rec->plan);
  rec->magic = 0;
  delete rec;
}
