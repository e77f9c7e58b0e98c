// Exact-integer twiddle factors (host side).
//
// Restates lean-fftw `LeanFFTW/Core/Trig.lean:25-134` in C++: cos/sin(2*pi*k/n) summed as
// Taylor series in 160-bit fixed point after an exact octant reduction of k/n, rounded to
// the nearest binary64, ties to even.  No libm call is made, so the tables are bit-identical
// to the reference's on every host (x86-64 and aarch64 alike).
#pragma once
#include <cstddef>
#include <cstdint>
#include <vector>

namespace lfg {

// (cos, sin)(2*pi*k/n) as binary64, n > 0 (Trig.lean:126).
void cos_sin_2pi(uint64_t k, uint64_t n, double* c, double* s);

// Table m -> (cos, sin)(2*pi*m/n), m < n, interleaved [c0, s0, c1, s1, ...]
// (Trig.lean:131-134; only n/gcd(8,n)+1 reduced angles are evaluated).
std::vector<double> cos_sin_2pi_table(uint64_t n);

// Twiddles of one Stockham pass (R, ns) of a size-N plan from the table `tab` of size N:
// for r = 1..R-1 the ns real parts, then the ns imaginary parts, of tab[r*k*N/(ns*R)];
// imaginary parts negated (never to -0.0) for forward transforms
// (lean-fftw `LeanFFTW/Core/FastPlan.lean:163-173`).
void pass_twiddles(const std::vector<double>& tab, bool fwd, uint64_t N, int R, uint64_t ns,
                   double* out);

}  // namespace lfg
