// The opaque plan handles of the C ABI (include/lfg.h) and the shared error message.
#pragma once
#include <exception>
#include <new>
#include <string>

#include "../../include/lfg.h"
#include "plan.h"
#include "ragged.h"

struct lfg_plan {
  lfg::Plan p;
};

struct lfg_ragged {
  lfg::RaggedPlan r;
};

namespace lfg {
// Message returned by lfg_last_error() on the calling thread.
void set_last_error(const std::string& msg);

// Runs an entry point's body, turning C++ exceptions (host allocation failures, library
// errors) into a status, so that none crosses the C ABI.
template <class F>
lfg_status guarded(F&& body) {
  try {
    return body();
  } catch (const std::bad_alloc&) {
    set_last_error("host allocation failed");
    return LFG_ERR_NOMEM;
  } catch (const std::exception& e) {
    set_last_error(std::string("internal error: ") + e.what());
    return LFG_ERR_INVALID;
  } catch (...) {
    set_last_error("internal error");
    return LFG_ERR_INVALID;
  }
}
}  // namespace lfg
