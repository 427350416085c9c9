"""CPU oracle for the TensorSat contraction path: TEST INFRASTRUCTURE ONLY.

A numpy restatement of the reference's arithmetic, used by ``tests/``, by
``__graft_entry__.smoke()`` and by ``bench.py``'s CPU-baseline leg to check and time the
GPU path. Nothing in the product package imports it; the product never falls back to it.

Restated functions (paths relative to the tensorsat project root):

* :func:`safe_dtype`       ``_to_safe_contraction_dtype``  tensorsat/lang/fin_rel.py:145-159
* :func:`rewire_array`     ``rewire_array``                tensorsat/_utils/misc.py:104-123
* :func:`contract2_or_and` ``FinRel._contract2``           tensorsat/lang/fin_rel.py:255-288
  (``opt_einsum.contract`` on two operands is numpy's einsum with the same operands)
* :func:`rewire_or_and`    ``FinRel._rewire``              tensorsat/lang/fin_rel.py:379-393
* :func:`spider`           ``FinRel._spider``              tensorsat/lang/fin_rel.py:290-298
* :func:`simple_contract2_args` the ``contract2_args`` bookkeeping of
  ``SimpleContraction._new``                              tensorsat/contractions/simple.py:231-291
* :func:`tree_contract`    one ``contract2`` per tree node with cotengra-style wire
  bookkeeping (``CotengraContraction.contract`` -> ``tree.contract`` ->
  ``tensorsat/_autoray.py:31-62``), in the OR-AND semiring (SAT) or over exact integers
  (the unclamped einsum of the #SAT prototype notebook,
  notebooks/prototypes/2025-02-13-#sat-tensor-contraction.ipynb cells 9-12)
* :func:`brute_force_count` enumeration of all assignments (C, ``oracle/brute.c``)
* :func:`dpll_count`       exact model counting by DPLL search with unit propagation (C,
  ``oracle/dpll.c``), for instances beyond brute force

Parity status: SAT bits are pinned against the reference's own known-answer tests and
against outputs of the reference itself (fixtures in ``tests/golden``); per-step results
are pinned against ``FinRel._contract2`` outputs; model counts are pinned by brute force
and, beyond its reach, by the DPLL counter, itself checked against brute force (the
reference has no counting API).
"""

from __future__ import annotations

import ctypes
import os
import subprocess
from collections import Counter
from itertools import product
from math import prod
from pathlib import Path
from typing import Sequence

import numpy as np

ORACLE_DIR = Path(__file__).resolve().parent
BUILD_DIR = ORACLE_DIR / "_build"
BRUTE_LIB = BUILD_DIR / "libts_oracle.so"


# --------------------------------------------------------------------------------------
# per-step restatements


def safe_dtype(contraction_size: int, dtype: np.dtype) -> np.dtype:
    """dtype that cannot overflow when summing ``contraction_size`` products of 0/1
    entries (fin_rel.py:145-159)."""
    if contraction_size < 256:
        return dtype
    if contraction_size < 65536:
        return np.dtype("uint16")
    if contraction_size < 2**32:
        return np.dtype("uint32")
    return np.dtype("uint64")


def _einsum(lhs, lhs_wires, rhs, rhs_wires, out_wires):
    ids: dict[int, int] = {}
    for w in list(lhs_wires) + list(rhs_wires) + list(out_wires):
        ids.setdefault(w, len(ids))
    if len(ids) > 52:
        raise ValueError("oracle einsum supports at most 52 distinct wires per step")
    return np.einsum(lhs, [ids[w] for w in lhs_wires], rhs, [ids[w] for w in rhs_wires],
                     [ids[w] for w in out_wires])


def rewire_array(a: np.ndarray, out_ports: Sequence[int]) -> np.ndarray:
    """Rewires an array: output port i is input port out_ports[i]; repeated ports give
    the diagonal (zeros elsewhere), absent ports are summed (misc.py:104-123)."""
    a_ports = range(a.ndim)
    b = np.zeros(tuple(a.shape[p] for p in out_ports), dtype=a.dtype)
    loop_ports = sorted(p for p, c in Counter(out_ports).items() if c > 1)
    loop_ports += sorted(set(a_ports) - set(out_ports))
    where = {p: i for i, p in enumerate(loop_ports)}
    for vals in product(*(range(a.shape[p]) for p in loop_ports)):
        a_idx = tuple(vals[where[p]] if p in where else slice(None) for p in a_ports)
        b_idx = tuple(vals[where[p]] if p in where else slice(None) for p in out_ports)
        b[b_idx] += a[a_idx]
    return b


def contract2_or_and(lhs: np.ndarray, lhs_wires: Sequence[int], rhs: np.ndarray,
                     rhs_wires: Sequence[int], out_wires: Sequence[int]) -> np.ndarray:
    """FinRel._contract2: einsum over the widened operands, then sign, as uint8. The
    widening follows the reference exactly: only wires shared by both operands and absent
    from the output count towards the contraction size."""
    shared = (set(lhs_wires) & set(rhs_wires)) - set(out_wires)
    k = prod(d for d, w in zip(lhs.shape, lhs_wires) if w in shared)
    dt = safe_dtype(k, lhs.dtype)
    lt, rt = lhs.astype(dt), rhs.astype(dt)
    if len(set(out_wires)) == len(out_wires):
        return np.sign(_einsum(lt, lhs_wires, rt, rhs_wires, out_wires), dtype=np.uint8)
    uniq = sorted(set(out_wires))
    res = _einsum(lt, lhs_wires, rt, rhs_wires, uniq)
    res = rewire_array(res, [uniq.index(w) for w in out_wires])
    return np.sign(res, dtype=np.uint8)


def contract2_einsum_definition(lhs: np.ndarray, lhs_wires: Sequence[int], rhs: np.ndarray,
                                rhs_wires: Sequence[int], out_wires: Sequence[int]) -> np.ndarray:
    """The einsum-defined result of a pairwise contraction with sign: output port i
    carries wire out_wires[i]; ports sharing a wire form a diagonal (zero elsewhere).
    Upstream agrees with this except when repeated output wires are interleaved with
    others out of sorted order, where ``rewire_array`` transposes blocks or raises."""
    uniq = list(dict.fromkeys(out_wires))
    res = _einsum(lhs.astype(np.uint64), lhs_wires, rhs.astype(np.uint64), rhs_wires, uniq)
    out = np.zeros([res.shape[uniq.index(w)] for w in out_wires], dtype=np.uint8)
    for idx in np.ndindex(*out.shape):
        val: dict[int, int] = {}
        if all(val.setdefault(w, v) == v for w, v in zip(out_wires, idx)):
            out[idx] = 1 if res[tuple(val[w] for w in uniq)] else 0
    return out


def rewire_or_and(t: np.ndarray, out_ports: Sequence[int]) -> np.ndarray:
    """FinRel._rewire: transpose when out_ports is a permutation, otherwise
    duplicate/discard ports (summing discarded ones) and take the sign."""
    out_ports = list(out_ports)
    if len(set(out_ports)) == len(out_ports) == t.ndim:
        return np.transpose(t, out_ports).copy()
    discarded = set(range(t.ndim)) - set(out_ports)
    if discarded:
        k = prod(d for p, d in enumerate(t.shape) if p in discarded)
        t = t.astype(safe_dtype(k, t.dtype))
    return np.sign(rewire_array(t, out_ports), dtype=np.uint8)


def spider(dim: int, num_ports: int) -> np.ndarray:
    """FinRel._spider: 1 on the main diagonal, 0 elsewhere."""
    t = np.zeros((dim,) * num_ports, dtype=np.uint8)
    for i in range(dim):
        t[(i,) * num_ports] = 1
    return t


def contract2_count(lhs: np.ndarray, lhs_wires: Sequence[int], rhs: np.ndarray,
                    rhs_wires: Sequence[int], out_wires: Sequence[int]) -> np.ndarray:
    """Exact integer contraction (no sign): uint64 when provably safe, else Python ints."""
    out_wires = list(out_wires)
    uniq = list(dict.fromkeys(out_wires))
    summed = (set(lhs_wires) | set(rhs_wires)) - set(uniq)
    dims = dict(zip(lhs_wires, lhs.shape))
    dims.update(zip(rhs_wires, rhs.shape))
    terms = prod(dims[w] for w in summed)
    lmax = int(lhs.max()) if lhs.size else 0
    rmax = int(rhs.max()) if rhs.size else 0
    if lmax * rmax * terms < 2**63 and lhs.dtype != object and rhs.dtype != object:
        res = _einsum(lhs.astype(np.uint64), lhs_wires, rhs.astype(np.uint64), rhs_wires, uniq)
    else:
        res = _einsum(lhs.astype(object), lhs_wires, rhs.astype(object), rhs_wires, uniq)
    if uniq != out_wires:
        res = rewire_array(res, [uniq.index(w) for w in out_wires])
    return res


# --------------------------------------------------------------------------------------
# drivers


def simple_contract2_args(slot_wires_list, out_wires, path):
    """The (lhs_idx, lhs_wires, rhs_idx, rhs_wires, res_wires) tuples SimpleContraction
    computes for a pop/append path (simple.py:238-278)."""
    args = []
    wires_list = [tuple(ws) for ws in slot_wires_list]
    for li, ri in path:
        lw = wires_list.pop(li)
        rw = wires_list.pop(ri - int(li < ri))
        common = set(lw) & set(rw)
        if common:
            res = tuple(w for w in lw if w not in common) + tuple(w for w in lw if w in common) \
                + tuple(w for w in rw if w not in common)
        else:
            res = lw + rw
        wires_list.append(res)
        args.append([li, lw, ri, rw, list(res)])
    if args:
        final = args[-1][-1]
        for w in sorted(set(final) - set(out_wires)):
            for a in reversed(args):
                if w in a[4]:
                    a[4].remove(w)
                    break
    return [(a, aw, b, bw, tuple(r)) for a, aw, b, bw, r in args]


def tree_contract(arrays: Sequence[np.ndarray], leaf_wires: Sequence[Sequence[int]],
                  out_wires: Sequence[int], steps: Sequence[tuple[int, int]],
                  semiring: str = "or_and", fixed: dict[int, int] | None = None) -> np.ndarray:
    """Contracts leaves along an SSA tree (step s makes node len(leaves)+s from
    steps[s]); a wire is summed at the first step after which no remaining tensor and no
    output needs it. ``fixed`` slices wires (leaves are indexed at the given values).
    Returns the result with axes in ``out_wires`` order (repeats -> diagonal)."""
    fixed = fixed or {}
    nodes: dict[int, tuple[np.ndarray, tuple[int, ...]]] = {}
    for i, (a, ws) in enumerate(zip(arrays, leaf_wires)):
        a = np.asarray(a)
        ws = tuple(ws)
        if fixed:
            idx = tuple(fixed[w] if w in fixed else slice(None) for w in ws)
            a = a[idx]
            ws = tuple(w for w in ws if w not in fixed)
        if semiring == "count":
            a = a.astype(np.uint64)
        nodes[i] = (a, ws)
    uniq_out = list(dict.fromkeys(out_wires))
    holders = Counter(w for _, ws in nodes.values() for w in set(ws))
    L = len(arrays)
    for s, (x, y) in enumerate(steps):
        (a, aw), (b, bw) = nodes.pop(x), nodes.pop(y)
        for w in set(aw):
            holders[w] -= 1
        for w in set(bw):
            holders[w] -= 1
        keep = [w for w in dict.fromkeys(aw + bw) if holders[w] > 0 or w in uniq_out]
        if semiring == "or_and":
            res = contract2_or_and(a, aw, b, bw, keep)
        else:
            res = contract2_count(a, aw, b, bw, keep)
        for w in keep:
            holders[w] += 1
        nodes[L + s] = (res, tuple(keep))
    (res, rw), = nodes.values()
    extra = [w for w in rw if w not in uniq_out]
    if extra:
        raise ValueError("root carries wires outside the output")
    order = [rw.index(w) for w in uniq_out]
    res = np.transpose(res, order) if order else res
    if list(uniq_out) != list(out_wires):
        res = rewire_array(res, [uniq_out.index(w) for w in out_wires])
    return res


# --------------------------------------------------------------------------------------
# brute force (C)


def build_oracle(force: bool = False) -> Path:
    """Compiles oracle/brute.c and oracle/dpll.c into oracle/_build/libts_oracle.so with
    gcc."""
    srcs = [ORACLE_DIR / "brute.c", ORACLE_DIR / "dpll.c"]
    if BRUTE_LIB.exists() and not force and \
            BRUTE_LIB.stat().st_mtime >= max(src.stat().st_mtime for src in srcs):
        return BRUTE_LIB
    BUILD_DIR.mkdir(exist_ok=True)
    cc = os.environ.get("CC", "gcc")
    tmp = BRUTE_LIB.with_suffix(".so.tmp")
    subprocess.run([cc, "-O2", "-shared", "-fPIC", "-o", str(tmp)] + [str(x) for x in srcs],
                   check=True)
    os.replace(tmp, BRUTE_LIB)
    return BRUTE_LIB


_brute = None


def brute_force_count(num_vars: int, clauses: Sequence[Sequence[int]]) -> int:
    """Number of assignments of variables 1..num_vars satisfying every clause."""
    global _brute
    if _brute is None:
        lib = ctypes.CDLL(str(build_oracle()))
        lib.ts_oracle_brute_count.restype = ctypes.c_int64
        lib.ts_oracle_brute_count.argtypes = [ctypes.c_int32, ctypes.c_int32,
                                              ctypes.POINTER(ctypes.c_int32),
                                              ctypes.POINTER(ctypes.c_int32)]
        _brute = lib
    offsets = [0]
    lits: list[int] = []
    for c in clauses:
        lits.extend(c)
        offsets.append(len(lits))
    off = (ctypes.c_int32 * len(offsets))(*offsets)
    lt = (ctypes.c_int32 * max(1, len(lits)))(*lits)
    res = _brute.ts_oracle_brute_count(num_vars, len(clauses), off, lt)
    if res < 0:
        raise ValueError("brute force supports at most 40 variables")
    return int(res)


def _clause_arrays(clauses: Sequence[Sequence[int]]):
    offsets = [0]
    lits: list[int] = []
    for c in clauses:
        lits.extend(c)
        offsets.append(len(lits))
    return ((ctypes.c_int32 * len(offsets))(*offsets),
            (ctypes.c_int32 * max(1, len(lits)))(*lits))


def dpll_count(num_vars: int, clauses: Sequence[Sequence[int]],
               node_limit: int = 50_000_000) -> tuple[int, int]:
    """(number of assignments of variables 1..num_vars satisfying every clause, search
    nodes visited), by DPLL search with unit propagation (C, ``oracle/dpll.c``), exact
    below 2^128. Raises RuntimeError when the search exceeds ``node_limit`` or the count
    reaches 2^128."""
    lib = ctypes.CDLL(str(build_oracle()))
    fn = lib.ts_oracle_dpll_count
    fn.restype = ctypes.c_int32
    fn.argtypes = [ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(ctypes.c_int32),
                   ctypes.POINTER(ctypes.c_int32), ctypes.c_uint64,
                   ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64),
                   ctypes.POINTER(ctypes.c_uint64)]
    off, lt = _clause_arrays(clauses)
    hi, lo, nodes = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
    st = fn(num_vars, len(clauses), off, lt, node_limit, ctypes.byref(hi), ctypes.byref(lo),
            ctypes.byref(nodes))
    if st == -1:
        raise ValueError("bad DPLL arguments (variable count or literal out of range)")
    if st == -2:
        raise RuntimeError(f"DPLL search exceeded {node_limit} nodes")
    if st == -4:
        raise RuntimeError("model count is 2^128 or more")
    if st != 0:
        raise RuntimeError(f"DPLL counter failed with status {st}")
    return (hi.value << 64) | lo.value, nodes.value


# --------------------------------------------------------------------------------------
# CNF networks


def clause_tensor(clause: Sequence[int]) -> tuple[np.ndarray, tuple[int, ...]]:
    """The clause as a 0/1 tensor over its distinct variables (wire i = variable i+1):
    1 exactly at assignments satisfying some literal."""
    vs = list(dict.fromkeys(abs(l) - 1 for l in clause))
    r = len(vs)
    t = np.zeros((2,) * r, dtype=np.uint8)
    for idx in np.ndindex(*t.shape):
        val = dict(zip(vs, idx))
        t[idx] = 1 if any(val[abs(l) - 1] == (1 if l > 0 else 0) for l in clause) else 0
    return t, tuple(vs)


def cnf_count_by_tree(num_vars: int, clauses, steps, semiring: str = "count",
                      fixed: dict[int, int] | None = None):
    """Count (or SAT bit) of a CNF through its clause network along ``steps``; variables
    in no clause contribute a factor 2 each to counts."""
    arrays, wires = zip(*(clause_tensor(c) for c in clauses))
    res = tree_contract(list(arrays), list(wires), (), steps, semiring, fixed)
    used = {w for ws in wires for w in ws}
    free = num_vars - len(used)
    if semiring == "count":
        fixed_free = 0 if not fixed else len([w for w in fixed if w not in used])
        return int(res) * 2 ** (free - fixed_free)
    return int(res)
