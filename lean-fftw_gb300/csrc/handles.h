// The opaque plan handles of the C ABI (include/lfg.h) and the shared error message.
#pragma once
#include <string>

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
}  // namespace lfg
