// Device autotuner (tuner.cpp).
#pragma once
#include <string>
#include <vector>

#include "plan.h"
#include "ragged.h"

namespace lfg {

// Radix sequences (first radix untwiddled, then a non-increasing twiddled tail) whose codelet
// operation count is within `slack` of the fewest, cheapest first, at most max_count.
std::vector<std::vector<int>> candidate_radices(int64_t n, double slack, size_t max_count);

// Time candidate (radices, grouping, tile) configurations of a c2c plan whose size, batch and
// precision are set; on success p.radices, p.single_max and p.tile hold the fastest.
std::string tune_c2c(Plan& p, int64_t default_tile);

// Time block shape, tile size and single-group limit of a ragged batch on scratch buffers;
// on success `opt` holds the fastest.
std::string tune_ragged(RaggedPlan& r, RaggedOptions& opt);

// Tuning cache (tuner.cpp): both tuners consult it before timing anything and record what
// they choose.  Import merges a file's entries, export writes every entry, forget empties it.
bool wisdom_import(const char* path);
bool wisdom_export(const char* path);
void wisdom_forget();
size_t wisdom_size();

}  // namespace lfg
