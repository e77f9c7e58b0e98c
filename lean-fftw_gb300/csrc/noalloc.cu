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

// The two-group launch sequence of an in-place complex plan with a caller-given intermediate
// (contiguous lines of n elements); single-group plans need none.
cudaError_t run_inplace(const lfg::Plan& p, void* data, void* scratch, cudaStream_t stream) {
  const size_t es = p.precision == 0 ? 16 : 8;
  char* base = static_cast<char*>(data);
  const char* ib = base + p.in.offset * (int64_t)es;
  char* ob = base + p.out.offset * (int64_t)es;
  auto launch = [&](const lfg::GroupDesc& g, const void* a, void* b) -> cudaError_t {
    if (p.precision == 0) return lfg::launch_group_f64(g, p.fwd, a, b, stream);
    return lfg::launch_group_f32(g, p.fwd, a, b, stream);
  };
  if (p.ngroups == 1) return launch(p.groups[0], ib, ob);
  lfg::GroupDesc g1 = p.groups[0], g2 = p.groups[1];
  const int64_t P = g2.nsub;
  g1.out_line = p.n;
  g1.out_sub = P;
  g1.out_elem = 1;
  g2.in_line = p.n;
  g2.in_sub = 1;
  g2.in_elem = P;
  cudaError_t e = launch(g1, ib, scratch);
  if (e != cudaSuccess) return e;
  return launch(g2, scratch, ob);
}

}  // namespace

extern "C" lfg_status lfg_execute_inplace_static(const lfg_plan* plan, void* data, void* stream) {
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
  if ((uintptr_t)data & (p.precision == 0 ? 15u : 7u)) {
    lfg::set_last_error("buffer must be aligned to a complex element (16 bytes binary64, 8 bytes binary32)");
    return LFG_ERR_INVALID;
  }
  if (!p.stages.empty() || p.howmany2 > 1) {
    lfg::set_last_error("static-scratch execution takes 1-D plans with one batch dimension");
    return LFG_ERR_UNSUPPORTED;
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
  if (e == cudaSuccess) e = run_inplace(p, data, scratch, static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) {
    lfg::set_last_error(std::string("static-scratch execution: ") + cudaGetErrorString(e));
    return LFG_ERR_CUDA;
  }
  return LFG_OK;
}
