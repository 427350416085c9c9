// Host-side planner kernel of the tensorsat_gb300 library: the dynamic program over
// subsets that subtree reconfiguration (tensorsat_gb300/planner.py, `reconfigure`) runs
// for every subtree it cuts. No device code: the planner stands in for the contraction-
// tree search the reference delegates to cotengra's hyper-optimiser
// (ctg.array_contract_tree, tensorsat/contractions/cotengra.py:78-85).
#include <stdint.h>

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "tsg_common.cuh"

namespace {

inline int popcount_words(const uint64_t* x, const uint64_t* y, const uint64_t* mask,
                          int words) {
  int c = 0;
  for (int w = 0; w < words; ++w) c += __builtin_popcountll((x[w] | y[w]) & mask[w]);
  return c;
}

}  // namespace

extern "C" tsg_status tsg_plan_subset_dp(int32_t n, int32_t words, const uint64_t* bits,
                                         const uint64_t* keep, const uint64_t* live,
                                         int32_t max_bits, double* best_full,
                                         uint32_t* split, uint64_t* kept) {
  if (n < 1 || n > 20 || words < 1 || words > 64)
    return tsg::fail(TSG_ERR_INVALID_ARGUMENT,
                     "tsg_plan_subset_dp: n must be in [1, 20] and words in [1, 64]");
  if (!bits || !keep || !live || !best_full || !split || !kept)
    return tsg::fail(TSG_ERR_INVALID_ARGUMENT, "tsg_plan_subset_dp: null argument");
  const uint32_t full = (1u << n) - 1u;
  const size_t W = (size_t)words;
  // union[m]: wires of the inputs in m; kept[m]: those that m's partial contraction keeps
  // (the subtree root keeps them, or an input outside m carries them)
  std::vector<uint64_t> uni((size_t)(full + 1) * W, 0);
  for (uint32_t m = 1; m <= full; ++m) {
    const uint32_t low = m & (0u - m);
    const int i = __builtin_ctz(low);
    const uint64_t* a = &uni[(size_t)(m ^ low) * W];
    uint64_t* u = &uni[(size_t)m * W];
    for (size_t w = 0; w < W; ++w) u[w] = a[w] | bits[(size_t)i * W + w];
  }
  std::memset(kept, 0, sizeof(uint64_t) * W);
  for (uint32_t m = 1; m <= full; ++m) {
    const uint64_t* u = &uni[(size_t)m * W];
    const uint64_t* c = &uni[(size_t)(full ^ m) * W];
    uint64_t* k = &kept[(size_t)m * W];
    for (size_t w = 0; w < W; ++w) k[w] = u[w] & (keep[w] | c[w]);
  }
  const double inf = INFINITY;
  std::vector<double> best((size_t)full + 1, 0.0);
  std::memset(split, 0, sizeof(uint32_t) * ((size_t)full + 1));
  for (uint32_t m = 1; m <= full; ++m) {
    if ((m & (m - 1)) == 0) continue;  // one input: no step
    const uint64_t* km = &kept[(size_t)m * W];
    if (m != full && max_bits >= 0 && popcount_words(km, km, live, words) > max_bits) {
      best[m] = inf;  // intermediate above the cap
      continue;
    }
    const uint32_t low = m & (0u - m);
    const uint32_t rest = m ^ low;
    double top = inf;
    uint32_t sub = rest;
    for (;;) {  // A = low | sub (holds the lowest input), B = the rest, sub descending
      const uint32_t a = low | sub;
      const uint32_t b = m ^ a;
      if (b) {
        const int e = popcount_words(&kept[(size_t)a * W], &kept[(size_t)b * W], live, words);
        const double c = best[a] + best[b] + std::ldexp(1.0, e);
        if (c < top) {
          top = c;
          split[m] = a;
        }
      }
      if (sub == 0) break;
      sub = (sub - 1) & rest;
    }
    best[m] = top;
  }
  *best_full = best[full];
  return TSG_OK;
}
