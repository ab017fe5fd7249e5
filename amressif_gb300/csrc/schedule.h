// Checkpoint schedule of the adjoint sweeps (2D and 3D).
//
// Cost model of the reversal of a segment of l steps with s free snapshot
// slots, the u* of its last step at hand: a full step costs 1, a
// predictor-only run kPredCost. With no free slot the steps l-2 .. 0 are
// reached from the segment's first state (restore, advance, predictor):
//   T(l, 0) = (l-1)(l-2)/2 + (l-1) kPredCost,
//   T(l, s) = min_m  m + T(l-m, s-1) + T(m, s)
// (advance m steps and keep that level, reverse the right part, release the
// slot, reverse the left part). Solved by dynamic programming when s L^2 is
// small, else Griewank's binomial split: with r the least repetition number
// for which beta(s, r) >= l, the right part gets min(l-1, beta(s-1, r)) steps.
#pragma once
#include <algorithm>
#include <vector>

namespace nsh {

constexpr double kPredCost = 0.75;

// binomial coefficient C(s + r, s), saturated
inline long long binomial_beta(int s, int r) {
  double b = 1.0;
  for (int k = 1; k <= s; ++k) {
    b = b * (double)(r + k) / (double)k;
    if (b > 4.0e18) return (long long)4.0e18;
  }
  return (long long)(b + 0.5);
}

struct Schedule {
  std::vector<int> split_arg;  // (s, l) -> steps to advance before the next snapshot; 0: no split
  int S = -1, L = -1;

  void build(int nsteps, int free_slots) {
    const int Sx = std::max(0, std::min(free_slots, nsteps - 1));
    if (L == nsteps && S == Sx) return;
    L = nsteps;
    S = Sx;
    split_arg.clear();
    if ((double)S * L * L > 3.0e8 || S == 0) return;
    std::vector<double> T((size_t)(S + 1) * (L + 1), 0.0);
    split_arg.assign((size_t)(S + 1) * (L + 1), 0);
    auto at = [&](int s, int l) -> double& { return T[(size_t)s * (L + 1) + l]; };
    for (int l = 1; l <= L; ++l) at(0, l) = 0.5 * (l - 1) * (l - 2) + (l - 1) * kPredCost;
    for (int s = 1; s <= S; ++s) {
      at(s, 1) = 0.0;
      for (int l = 2; l <= L; ++l) {
        double best = at(0, l);
        int arg = 0;
        for (int m = 1; m < l; ++m) {
          const double v = m + at(s - 1, l - m) + at(s, m);
          if (v < best) { best = v; arg = m; }
        }
        at(s, l) = best;
        split_arg[(size_t)s * (L + 1) + l] = arg;
      }
    }
  }

  // next snapshot of the segment [a, b) with s free slots; -1: reverse it from a
  int next(int a, int b, int s) const {
    const int l = b - a;
    if (s <= 0 || l < 2) return -1;
    if (!split_arg.empty() && l <= L) {
      const int m = split_arg[(size_t)std::min(s, S) * (L + 1) + l];
      return m > 0 ? a + m : -1;
    }
    int r = 1;
    while (binomial_beta(s, r) < l) ++r;
    const long long right = std::min((long long)l - 1, binomial_beta(s - 1, r));
    return b - (int)right;
  }
};

}  // namespace nsh
