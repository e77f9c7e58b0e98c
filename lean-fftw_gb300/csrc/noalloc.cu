// In-place execution without any allocation: the intermediate of two-group complex plans
// lives in a fixed, file-scope device array instead of plan-owned memory.
//
// lfg_execute allocates the plan's scratch buffer with cudaMalloc the first time an in-place
// two-group plan runs.  Some callers cannot allow that: frameworks that route every device
// allocation through their own pool and forbid direct cudaMalloc (so their accounting of
// device memory stays exact), and steady-state loops that cannot take cudaMalloc's implicit
// device-wide synchronisation.  lfg_execute_inplace_static serves them: it calls no cudaMalloc,
// cudaFree or allocating library routine; the plan (created earlier) owns only its twiddle
// tables.
//
// The array holds kStaticScratchBytes (16 MiB); every GPU that loads this library keeps it
// until the process exits.  In host code `g_static_scratch` names a host-side stand-in, not a
// device address, so its device address is looked up once per device with
// cudaGetSymbolAddress (on the first call on that device, with the device current) and that
// address is passed to the kernels.  All calls share the one array and it keeps the contents
// of the last call; the kernels overwrite every element they later read, so nothing needs
// clearing, but two calls whose executions overlap on the GPU race on it.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <string>

#include "../../include/lfg.h"
#include "kernels.h"
#include "plan.h"

#include "handles.h"

namespace {

constexpr size_t kStaticScratchBytes = (size_t)16 << 20;

static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
void* g_scratch_addr[kMaxDevices] = {};

// Device address of the static array on the current device (looked up once per device).
cudaError_t static_scratch(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_mutex);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_static_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return cudaSuccess;
}

lfg_status execute_inplace_static(const lfg_plan* plan, void* data, void* stream) {
  if (!plan || !data) {
    lfg::set_last_error("null plan or buffer");
    return LFG_ERR_INVALID;
  }
  const lfg::Plan& p = plan->p;
  if (p.kind != lfg::Kind::C2C) {
    lfg::set_last_error("static-scratch execution takes complex (c2c) plans only");
    return LFG_ERR_UNSUPPORTED;
  }
  if (p.empty) return LFG_OK;
  // only plans that run as one or two pass groups of the Stockham kernels: sizes with a prime
  // factor above 13 (generic-engine and Bluestein plans) and dense-buffer plans (split arrays,
  // negative strides) keep buffers of their own and are refused before anything runs
  if (p.generic || p.chirp_fwd || !p.steps.empty() || (p.ngroups != 1 && p.ngroups != 2)) {
    lfg::set_last_error("static-scratch execution takes 13-smooth sizes in one or two pass "
                        "groups only (this plan runs another algorithm)");
    return LFG_ERR_UNSUPPORTED;
  }
  if (!p.stages.empty() || p.howmany2 > 1) {
    lfg::set_last_error("static-scratch execution takes 1-D plans with one batch dimension");
    return LFG_ERR_UNSUPPORTED;
  }
  if ((uintptr_t)data & (p.precision == 0 ? 15u : 7u)) {
    lfg::set_last_error("buffer must be aligned to a complex element (16 bytes binary64, 8 bytes binary32)");
    return LFG_ERR_INVALID;
  }
  const size_t es = p.precision == 0 ? 16 : 8;
  const size_t need = (size_t)p.n * (size_t)p.howmany * es;
  if (p.ngroups == 2 && need > kStaticScratchBytes) {
    lfg::set_last_error("intermediate of " + std::to_string(need) + " bytes exceeds the " +
                        std::to_string(kStaticScratchBytes) + "-byte static scratch array");
    return LFG_ERR_UNSUPPORTED;
  }
  void* scratch = nullptr;
  cudaError_t e = p.ngroups == 2 ? static_scratch(&scratch) : cudaSuccess;
  // the regular launch sequence, in place, with the static array as the two-group
  // intermediate (a one-group plan needs none)
  if (e == cudaSuccess)
    e = lfg::execute_plan(p, data, data, static_cast<cudaStream_t>(stream), false, scratch);
  if (e != cudaSuccess) {
    lfg::set_last_error(std::string("static-scratch execution: ") + cudaGetErrorString(e));
    return LFG_ERR_CUDA;
  }
  return LFG_OK;
}

}  // namespace

extern "C" lfg_status lfg_execute_inplace_static(const lfg_plan* plan, void* data, void* stream) {
  return lfg::guarded([&] { return execute_inplace_static(plan, data, stream); });
}
