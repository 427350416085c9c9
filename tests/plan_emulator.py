"""Numpy emulation of the tree executor's index semantics (test infrastructure).

Given the integer arrays a :class:`tensorsat_gb300.planner.SlicedPlan` emits for
``tsg_plan_create`` and the flattened uint8 leaves, computes the per-slice root tensors
exactly as the header ``include/tensorsat_gb300.h`` specifies them: step ``s`` maps output
bit ``i`` / summed bit ``j`` to the operand bit positions in ``step_lhs_pos`` /
``step_rhs_pos``, and sliced wires of leaves are fixed from the slice id. This pins the
planner's arrays on the CPU, independently of the CUDA code.
"""

from __future__ import annotations

import numpy as np


def _gather_offsets(pos_row, out_bits, k_bits):
    t = np.arange(1 << out_bits, dtype=np.int64)[:, None]
    k = np.arange(1 << k_bits, dtype=np.int64)[None, :]
    off = np.zeros((1 << out_bits, 1 << k_bits), dtype=np.int64)
    for i in range(out_bits):
        p = pos_row[i]
        if p >= 0:
            off |= ((t >> i) & 1) << p
    for j in range(k_bits):
        p = pos_row[out_bits + j]
        if p >= 0:
            off |= ((k >> j) & 1) << p
    return off


def emulate(arrs: dict, leaves: list[np.ndarray], slice_id: int, semiring: str) -> np.ndarray:
    """Root tensor (flat, 2^root_bits entries) of one slice; counts as Python ints."""
    L = len(leaves)
    spos = arrs["leaf_slice_pos"]
    nsl = spos.shape[1]
    vals: dict[int, np.ndarray] = {}
    for l in range(L):
        flat = leaves[l].reshape(-1)
        vals[l] = flat.astype(object) if semiring == "count" else flat.astype(np.uint8)
    res = None
    for s in range(len(arrs["step_out_bits"])):
        ob = int(arrs["step_out_bits"][s])
        kb = int(arrs["step_sum_bits"][s])
        operands = []
        for o, key in enumerate(("step_lhs_pos", "step_rhs_pos")):
            v = int(arrs["step_operands"][s, o])
            node = v if v >= 0 else L + (-v - 1)
            off = _gather_offsets(arrs[key][s], ob, kb)
            if v >= 0:
                for j in range(nsl):
                    p = spos[v, j]
                    if p >= 0:
                        off = off | (((slice_id >> j) & 1) << int(p))
            operands.append(vals[node][off])
        if semiring == "count":
            out = (operands[0] * operands[1]).sum(axis=1)
        else:
            out = (operands[0] & operands[1]).max(axis=1).astype(np.uint8)
        vals[L + s] = out
        res = out
    return res


def emulate_all(arrs: dict, leaves: list[np.ndarray], semiring: str) -> np.ndarray:
    nsl = arrs["leaf_slice_pos"].shape[1]
    total = None
    for sid in range(1 << nsl):
        r = emulate(arrs, leaves, sid, semiring)
        if total is None:
            total = r
        elif semiring == "count":
            total = total + r
        else:
            total = np.maximum(total, r)
    return total
