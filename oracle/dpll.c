/*
 * Exact model counter for CNF formulas by DPLL search: test infrastructure only (an
 * oracle that pins exact model counts beyond brute force, e.g. random 3-SAT n=60 or
 * 5-SAT n=39). It is never part of the product path.
 *
 * The count is the full unclamped contraction of the CNF network (the #SAT prototype
 * notebook, notebooks/prototypes/2025-02-13-#sat-tensor-contraction.ipynb cells 9-12),
 * computed here without any tensor network: the search splits on one variable at a time,
 * propagates unit clauses, returns 0 on an empty clause and 2^(unassigned variables) once
 * every clause is satisfied. The counts of the two branches add up, so the total is the
 * number of satisfying assignments of the n variables. The branching variable comes from
 * an unsatisfied clause with the fewest unassigned literals.
 */
#include <stdint.h>
#include <stdlib.h>

typedef struct {
  int32_t n, m;
  const int32_t* off;
  const int32_t* lit;
  int8_t* val;       /* per variable: -1 unassigned, 0, 1 */
  int32_t* trail;    /* assigned variables, in order */
  int32_t ntrail;
  uint64_t nodes;    /* search nodes visited */
  uint64_t node_limit;
  int aborted;       /* 1: node limit reached, 2: count at or above 2^128 */
} Search;

/* 1 if the literal is true under the current assignment, 0 if false, -1 if unassigned */
static int lit_value(const Search* s, int32_t l) {
  const int32_t v = (l > 0 ? l : -l) - 1;
  const int8_t x = s->val[v];
  if (x < 0) return -1;
  return (l > 0) == (x == 1);
}

static void assign(Search* s, int32_t v, int8_t x) {
  s->val[v] = x;
  s->trail[s->ntrail++] = v;
}

static void undo(Search* s, int32_t mark) {
  while (s->ntrail > mark) s->val[s->trail[--s->ntrail]] = -1;
}

/* Unit propagation to a fixed point. Returns 0 on a conflict, 1 otherwise; *open_clause
 * receives an unsatisfied clause with the fewest unassigned literals (-1: all satisfied). */
static int propagate(Search* s, int32_t* open_clause) {
  for (;;) {
    int changed = 0;
    int32_t best = -1, best_free = 1 << 30;
    for (int32_t c = 0; c < s->m; ++c) {
      int32_t free_lits = 0, unit = 0, sat = 0;
      for (int32_t j = s->off[c]; j < s->off[c + 1]; ++j) {
        const int x = lit_value(s, s->lit[j]);
        if (x == 1) {
          sat = 1;
          break;
        }
        if (x < 0) {
          /* a repeated literal counts once */
          if (free_lits == 0 || s->lit[j] != unit) ++free_lits;
          unit = s->lit[j];
        }
      }
      if (sat) continue;
      if (free_lits == 0) return 0;
      if (free_lits == 1) {
        const int32_t v = (unit > 0 ? unit : -unit) - 1;
        assign(s, v, unit > 0 ? 1 : 0);
        changed = 1;
        continue;
      }
      if (free_lits < best_free) {
        best_free = free_lits;
        best = c;
      }
    }
    if (!changed) {
      *open_clause = best;
      return 1;
    }
  }
}

/* number of satisfying extensions of the current assignment, as (hi, lo) 128-bit */
static void count_rec(Search* s, uint64_t* hi, uint64_t* lo) {
  *hi = 0;
  *lo = 0;
  if (s->aborted) return;
  if (++s->nodes > s->node_limit) {
    s->aborted = 1;
    return;
  }
  const int32_t mark = s->ntrail;
  int32_t c = -1;
  if (!propagate(s, &c)) {
    undo(s, mark);
    return;
  }
  if (c < 0) {
    const int32_t free_vars = s->n - s->ntrail;
    if (free_vars >= 128) s->aborted = 2;
    else if (free_vars >= 64) *hi = (uint64_t)1 << (free_vars - 64);
    else *lo = (uint64_t)1 << free_vars;
    undo(s, mark);
    return;
  }
  int32_t v = -1;
  for (int32_t j = s->off[c]; j < s->off[c + 1] && v < 0; ++j)
    if (lit_value(s, s->lit[j]) < 0) v = (s->lit[j] > 0 ? s->lit[j] : -s->lit[j]) - 1;
  for (int8_t x = 0; x < 2; ++x) {
    const int32_t m2 = s->ntrail;
    assign(s, v, x);
    uint64_t h, l;
    count_rec(s, &h, &l);
    undo(s, m2);
    *lo += l;
    const uint64_t carry = *lo < l;
    const uint64_t h0 = *hi;
    *hi += h + carry;
    if (*hi < h0 || (carry && h == UINT64_MAX)) s->aborted = 2;
  }
  undo(s, mark);
}

/* Clause c spans lits[offsets[c] .. offsets[c+1]) (non-zero DIMACS literals over
 * variables 1..n). Writes the number of satisfying assignments as two 64-bit halves and
 * the number of search nodes visited. Returns 0 on success, -1 for bad arguments (n
 * outside [0, 10000], a literal out of range), -2 when the search visited more than
 * node_limit nodes, -3 when memory ran out, -4 when the count is 2^128 or more. */
int32_t ts_oracle_dpll_count(int32_t n, int32_t num_clauses, const int32_t* offsets,
                             const int32_t* lits, uint64_t node_limit, uint64_t* count_hi,
                             uint64_t* count_lo, uint64_t* nodes) {
  if (n < 0 || n > 10000 || num_clauses < 0) return -1;
  for (int32_t j = 0; j < (num_clauses ? offsets[num_clauses] : 0); ++j)
    if (lits[j] == 0 || lits[j] > n || lits[j] < -n) return -1;
  Search s;
  s.n = n;
  s.m = num_clauses;
  s.off = offsets;
  s.lit = lits;
  s.val = (int8_t*)malloc((size_t)(n > 0 ? n : 1));
  s.trail = (int32_t*)malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
  if (!s.val || !s.trail) {
    free(s.val);
    free(s.trail);
    return -3;
  }
  for (int32_t v = 0; v < n; ++v) s.val[v] = -1;
  s.ntrail = 0;
  s.nodes = 0;
  s.node_limit = node_limit;
  s.aborted = 0;
  uint64_t hi = 0, lo = 0;
  count_rec(&s, &hi, &lo);
  *count_hi = hi;
  *count_lo = lo;
  *nodes = s.nodes;
  free(s.val);
  free(s.trail);
  if (s.aborted == 1) return -2;
  if (s.aborted == 2) return -4;
  return 0;
}
