/*
 * Brute-force model counter for CNF formulas: test infrastructure only (the oracle that
 * pins exact model counts for n <= 30). It is never part of the product path.
 *
 * Bit-sliced enumeration: the 64 lanes of a word hold the 64 assignments that differ in
 * variables 0..5 (fixed bit patterns); the remaining variables take the value of the word
 * counter's bits. A clause evaluates as the OR of its literal words, the formula as the
 * AND of its clauses, and the count adds the popcount of the surviving lanes.
 *
 * The SAT bit this yields is the reference semantics of a closed CNF network contracted
 * to a scalar (tensorsat/lang/fin_rel.py:472-473 reads it as "scalar == 1"); the count is
 * the full unclamped contraction of the same network (the #SAT prototype notebook,
 * notebooks/prototypes/2025-02-13-#sat-tensor-contraction.ipynb cells 9-12).
 */
#include <stdint.h>

static const uint64_t kLanePattern[6] = {
    0xAAAAAAAAAAAAAAAAull, 0xCCCCCCCCCCCCCCCCull, 0xF0F0F0F0F0F0F0F0ull,
    0xFF00FF00FF00FF00ull, 0xFFFF0000FFFF0000ull, 0xFFFFFFFF00000000ull,
};

/* literals: clause c spans lits[offsets[c] .. offsets[c+1]), each a non-zero DIMACS
 * literal over variables 1..n. Returns the number of satisfying assignments of the n
 * variables, or -1 if n is outside [0, 40]. */
int64_t ts_oracle_brute_count(int32_t n, int32_t num_clauses, const int32_t* offsets,
                              const int32_t* lits) {
  if (n < 0 || n > 40) return -1;
  const int lane_vars = n < 6 ? n : 6;
  const uint64_t lane_mask = lane_vars == 6 ? ~0ull : ((1ull << (1u << lane_vars)) - 1ull);
  const int64_t words = (int64_t)1 << (n - lane_vars);
  int64_t total = 0;
  for (int64_t wi = 0; wi < words; ++wi) {
    uint64_t alive = lane_mask;
    for (int32_t c = 0; c < num_clauses && alive; ++c) {
      uint64_t sat = 0;
      for (int32_t j = offsets[c]; j < offsets[c + 1]; ++j) {
        const int32_t lit = lits[j];
        const int32_t v = (lit > 0 ? lit : -lit) - 1;
        uint64_t val;
        if (v < lane_vars) {
          val = kLanePattern[v];
        } else {
          val = ((wi >> (v - lane_vars)) & 1) ? ~0ull : 0ull;
        }
        sat |= lit > 0 ? val : ~val;
      }
      alive &= sat;
    }
    total += __builtin_popcountll(alive & lane_mask);
  }
  return total;
}
