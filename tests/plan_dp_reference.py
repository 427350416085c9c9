"""Pure-Python restatement of the planner's subset dynamic program (test infrastructure).

The native ``tsg_plan_subset_dp`` (``tensorsat_gb300/csrc/tsg_plan.cu``) must return
exactly what this returns: the same cost (the same double-precision sums in the same
order), the same split of every subset (the same visiting order, strict improvement
only) and the same kept wires. Wire sets are Python ints.
"""

from __future__ import annotations

from typing import Sequence


def subset_dp_reference(n: int, bits: Sequence[int], keep: int, live: int,
                        max_bits: int | None) -> tuple[float, list[int], list[int]]:
    full = (1 << n) - 1
    union = [0] * (full + 1)
    for m in range(1, full + 1):
        low = m & -m
        union[m] = union[m ^ low] | bits[low.bit_length() - 1]
    kept = [union[m] & (keep | union[full ^ m]) for m in range(full + 1)]
    inf = float("inf")
    best = [0.0] * (full + 1)
    split = [0] * (full + 1)
    for m in range(1, full + 1):
        if m & (m - 1) == 0:
            continue
        if m != full and max_bits is not None and (kept[m] & live).bit_count() > max_bits:
            best[m] = inf
            continue
        low = m & -m
        rest = m ^ low
        top = inf
        sub = rest
        while True:
            a = low | sub
            b = m ^ a
            if b:
                c = best[a] + best[b] + 2.0 ** ((kept[a] | kept[b]) & live).bit_count()
                if c < top:
                    top, split[m] = c, a
            if sub == 0:
                break
            sub = (sub - 1) & rest
        best[m] = top
    return best[full], split, kept


def slice_tree_reference(tree, target_bits: int, forbid=frozenset()):
    """Set-based restatement of the planner's greedy slicing (one full cost evaluation
    per candidate wire): the vectorised ``planner.slice_tree`` must pick the same wires."""
    sliced = set()
    L = tree.num_leaves
    while True:
        tot, peak, _ = tree.cost(frozenset(sliced))
        if peak <= target_bits:
            return frozenset(sliced)
        cands = set()
        for s in range(len(tree.steps)):
            ws = tree.node_wires[L + s] - sliced
            if len(ws) == peak:
                cands |= ws
        cands -= forbid
        if not cands:
            raise ValueError("cannot slice")
        best = None
        for w in sorted(cands):
            t2, p2, _ = tree.cost(frozenset(sliced | {w}))
            key = (p2, t2 + len(sliced) + 1)
            if best is None or key < best[0]:
                best = (key, w)
        sliced.add(best[1])


def unslice_reference(tree, sliced, target_bits: int):
    sl = set(sliced)
    for w in sorted(sliced):
        if tree.cost(frozenset(sl - {w}))[1] <= target_bits:
            sl.discard(w)
    return frozenset(sl)
