"""C ABI checks that need no GPU: the library loads, exports every declared symbol,
validates plans and arguments, and bounds-checks every launch of real plans."""

from __future__ import annotations

import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

from tensorsat_gb300 import _native, planner
from tensorsat_gb300.contractions.gpu import PRIMES_31, GpuContraction, NativePlan
from tensorsat_gb300.lang.cuda_rel import CudaRel
from tensorsat_gb300.lib.sat import CNFInstance

HEADER = Path(__file__).resolve().parent.parent / "include" / "tensorsat_gb300.h"


def declared_symbols() -> list[str]:
    text = HEADER.read_text()
    return re.findall(r"TSG_API\s+[\w\s\*]+?\b(tsg_\w+)\s*\(", text)


def test_library_exports_every_declared_symbol():
    lib = _native.lib()
    names = declared_symbols()
    assert len(names) >= 14
    assert set(names) == set(_native.EXPORTED_SYMBOLS)
    for name in names:
        assert hasattr(lib, name), name
    assert lib.tsg_abi_version() == 1


def test_null_arguments_are_rejected_without_touching_the_device():
    lib = _native.lib()
    st = lib.tsg_contract2_or_and(None, 0, None, None, None, 0, None, None, 0, None, None, None)
    assert st == _native.TSG_ERR_INVALID_ARGUMENT
    assert "null" in lib.tsg_last_error().decode()
    assert lib.tsg_union_or(None, None, None, -1, None) == _native.TSG_ERR_INVALID_ARGUMENT
    assert lib.tsg_spider_fill(None, 2, 2, None) == _native.TSG_ERR_INVALID_ARGUMENT
    assert lib.tsg_plan_run(None, 0, 0, None, None, 0, 1, 1, None, 0, None, 0, None) \
        == _native.TSG_ERR_INVALID_ARGUMENT


def _plan_for(cnf, target_bits, seed=0):
    d = cnf.clause_diagram()
    return GpuContraction(CudaRel, d.wiring, target_bits=target_bits, trials=2, seed=seed)


@pytest.mark.parametrize("n,m,target", [(12, 50, 4), (20, 85, 8), (30, 128, 14), (40, 170, 20)])
def test_every_launch_is_in_bounds(n, m, target):
    c = _plan_for(CNFInstance.random(3, n, m, rng=1), target)
    npl = c.native_plan()
    ns = c.num_slices
    for ring, primes in [(_native.TSG_RING_OR_AND, ()), (_native.TSG_RING_U64, ()),
                         (_native.TSG_RING_MODP, PRIMES_31[:3])]:
        for g in sorted({1, 2, min(16, ns), ns}):
            npl.validate(ring, primes, 0, ns, g)
        if ns >= 4:
            npl.validate(ring, primes, 2, ns - 1, 2)


def test_workspace_grows_with_group_and_ring():
    c = _plan_for(CNFInstance.random(3, 30, 128, rng=0), 12)
    npl = c.native_plan()
    w1 = npl.workspace_bytes(_native.TSG_RING_OR_AND, 1, 1)
    w8 = npl.workspace_bytes(_native.TSG_RING_OR_AND, 1, 8)
    w8p = npl.workspace_bytes(_native.TSG_RING_MODP, 3, 8)
    assert w1 <= w8 <= w8p
    assert w8p >= 12 * 8 * 2 ** c.stats()["peak_bits"]
    assert npl.launch_count(0, c.num_slices, 8) > 0


def test_bad_ranges_and_rings_are_rejected():
    c = _plan_for(CNFInstance.random(3, 20, 85, rng=0), 8)
    npl = c.native_plan()
    ns = c.num_slices
    with pytest.raises(_native.TsgValueError):
        npl.validate(_native.TSG_RING_OR_AND, (), 0, ns + 1, 1)
    with pytest.raises(_native.TsgValueError):
        npl.validate(_native.TSG_RING_OR_AND, (), 1, ns, 2)  # begin not a group multiple
    with pytest.raises(_native.TsgValueError):
        npl.validate(_native.TSG_RING_OR_AND, (), 0, ns, 3)  # not a power of two
    with pytest.raises(_native.TsgValueError):
        npl.validate(_native.TSG_RING_MODP, (4,), 0, ns, 1)  # even modulus
    with pytest.raises(_native.TsgValueError):
        npl.validate(7, (), 0, ns, 1)


def _create(arrs, offsets=None):
    lib = _native.lib()
    ranks = arrs["leaf_ranks"]
    if offsets is None:
        offsets = np.cumsum([0] + [1 << int(r) for r in ranks[:-1]]).astype(np.int64)
    h = ctypes.c_void_p()
    lsp = np.ascontiguousarray(arrs["leaf_slice_pos"], dtype=np.int32)
    st = lib.tsg_plan_create(
        len(ranks), _native.ptr_i32(ranks), _native.ptr_i64(offsets), lsp.shape[1],
        _native.ptr_i32(lsp), len(arrs["step_out_bits"]),
        _native.ptr_i32(np.ascontiguousarray(arrs["step_operands"])),
        _native.ptr_i32(arrs["step_out_bits"]), _native.ptr_i32(arrs["step_sum_bits"]),
        _native.ptr_i32(arrs["step_lhs_pos"]), _native.ptr_i32(arrs["step_rhs_pos"]),
        ctypes.byref(h))
    if st == _native.TSG_OK:
        lib.tsg_plan_destroy(h)
    return st


def test_plan_create_rejects_malformed_trees():
    cnf = CNFInstance.random(3, 10, 30, rng=0)
    c = _plan_for(cnf, 5)
    good = c.sliced_plan.native_arrays()
    assert _create(good) == _native.TSG_OK

    def mutated(key, fn):
        arrs = {k: v.copy() for k, v in good.items()}
        fn(arrs[key])
        return _create(arrs)

    # a leaf used twice
    assert mutated("step_operands", lambda a: a.__setitem__((1, 0), a[0, 0])) \
        == _native.TSG_ERR_INVALID_ARGUMENT
    # a step reading a later step
    assert mutated("step_operands", lambda a: a.__setitem__((0, 1), -3)) \
        == _native.TSG_ERR_INVALID_ARGUMENT
    # an operand bit left uncovered
    def drop_bit(a):
        s = int(np.argmax((a >= 0).sum(axis=1)))
        j = int(np.argmax(a[s] >= 0))
        a[s, j] = -1
    assert mutated("step_lhs_pos", drop_bit) == _native.TSG_ERR_INVALID_ARGUMENT
    # a bit position outside the operand
    assert mutated("step_rhs_pos", lambda a: a.__setitem__((0, 0), 61)) \
        == _native.TSG_ERR_INVALID_ARGUMENT
    # more index bits than the kernels address
    assert mutated("step_out_bits", lambda a: a.__setitem__(0, 70)) \
        == _native.TSG_ERR_INVALID_ARGUMENT


def test_native_plan_leaf_pool_layout():
    c = _plan_for(CNFInstance.random(3, 16, 60, rng=2), 6)
    npl = NativePlan(c.sliced_plan)
    offs = npl.leaf_offsets
    assert all(o % 16 == 0 for o in offs)
    assert all(offs[i] + npl.leaf_sizes[i] <= offs[i + 1] for i in range(len(offs) - 1))
    assert npl.pool_bytes >= offs[-1] + npl.leaf_sizes[-1]


def test_planner_native_arrays_shapes():
    cnf = CNFInstance.random(3, 14, 56, rng=4)
    d = cnf.clause_diagram()
    net = planner.Network([tuple(ws) for ws in d.wiring.slot_wires_list],
                          {w: 2 for w in range(14)}, ())
    tree, sl = planner.optimize(net, target_bits=5, trials=2)
    sp = planner.SlicedPlan(tree, tuple(sorted(sl)), list(net.leaf_wires))
    arrs = sp.native_arrays()
    assert arrs["step_lhs_pos"].shape == (len(tree.steps), planner.TSG_MAX_BITS)
    assert arrs["leaf_slice_pos"].shape == (len(net.leaf_wires), len(sl))


def test_kissat_and_benchmark_plans_validate_in_every_ring():
    """Bounds and vector-alignment proofs over every launch of real plans (gate networks
    of the known-answer set, the n=60 benchmark tree), all rings and several groups."""
    import json

    golden = Path(__file__).resolve().parent / "golden" / "kissat.json"
    for case in json.loads(golden.read_text())[::4] + [
            c for c in json.loads(golden.read_text()) if c["file"] == "prime121"]:
        cnf = CNFInstance(case["num_vars"], [tuple(c) for c in case["clauses"]])
        d = (cnf.inputs(None) >> cnf.diagram()).flatten()
        c = GpuContraction(CudaRel, d.wiring, trials=1)
        npl = c.native_plan()
        for ring, primes in [(_native.TSG_RING_OR_AND, ()), (_native.TSG_RING_MODP, PRIMES_31[:4]),
                             (_native.TSG_RING_U64, ())]:
            npl.validate(ring, primes, 0, c.num_slices, 1)
    cnf = CNFInstance.random(3, 60, 256, rng=0)
    c = GpuContraction(CudaRel, cnf.clause_diagram().wiring, target_bits=26, trials=2)
    npl = c.native_plan()
    for ring, primes in [(_native.TSG_RING_OR_AND, ()), (_native.TSG_RING_MODP, PRIMES_31[:3]),
                         (_native.TSG_RING_U64, ())]:
        for g in (1, 64):
            npl.validate(ring, primes, 0, 2 * g, g)


def _profiled_kernels():
    """(ring, step) -> (family, V, NE, NK) of every launch in the committed ncu summary of
    the n=60 benchmark tree (one MODP run with 3 primes and one OR-AND run, 64 slices)."""
    path = HEADER.parent.parent / "profiles" / "tree_steps_n60_dram.txt"
    rings = {"modp": _native.TSG_RING_MODP, "or_and": _native.TSG_RING_OR_AND}
    out = {}
    for line in path.read_text().splitlines():
        if line.startswith("#") or not line.strip():
            continue
        ring, step = line.split()[:2]
        m = re.search(r"tsg::(tree_step_\w+)<([^>]*)>", line)
        name, args = m.group(1), [int(x) for x in m.group(2).split(",")]
        if name == "tree_step_tile_kernel":
            kind = (_native.TSG_KERNEL_TILE, args[1], args[2], args[3])
        elif name == "tree_step_sum_kernel":
            kind = (_native.TSG_KERNEL_SUM, 0, 0, 0)
        elif name == "tree_step_fused_kernel":
            kind = (_native.TSG_KERNEL_FUSED, 4, args[1], args[2])
        elif name == "tree_step_stream_kernel":
            kind = (_native.TSG_KERNEL_STREAM, 0, args[1], args[2])
        else:
            kind = (_native.TSG_KERNEL_GENERAL, 0, 0, 0)
        out[(rings[ring], int(step))] = kind
    return out


def test_kernel_choice_matches_the_profiled_launches():
    """tsg_plan_describe reports, on the host, the kernel that ran for every step in the
    committed launch list of the benchmark (n=60, m=256, seed 0, 8 planner trials, 64
    slices per group): the host-side selection is the one the GPU executed."""
    cnf = CNFInstance.random(3, 60, 256, rng=0)
    c = GpuContraction(CudaRel, cnf.clause_diagram().wiring, target_bits=26, trials=8, seed=0)
    npl = c.native_plan()
    expected = _profiled_kernels()
    assert len(expected) >= 20
    lib = _native.lib()
    # the launch list records whether its run fused steps
    fused_run = any(kind[0] == _native.TSG_KERNEL_FUSED for kind in expected.values())
    lib.tsg_set_fusion(1 if fused_run else 0)
    try:
        got = {_native.TSG_RING_MODP: npl.describe(_native.TSG_RING_MODP, PRIMES_31[:3], 64),
               _native.TSG_RING_OR_AND: npl.describe(_native.TSG_RING_OR_AND, (), 64)}
    finally:
        lib.tsg_set_fusion(1)
    for (ring, step), kind in expected.items():
        assert tuple(int(x) for x in got[ring][step]) == kind, (ring, step)
    kinds = got[_native.TSG_RING_MODP][:, 0]
    assert set(kinds) <= {_native.TSG_KERNEL_GENERAL, _native.TSG_KERNEL_TILE,
                          _native.TSG_KERNEL_STREAM, _native.TSG_KERNEL_FUSED,
                          _native.TSG_KERNEL_NONE, _native.TSG_KERNEL_SUM}
    with pytest.raises(_native.TsgValueError):
        npl.describe(_native.TSG_RING_OR_AND, (), c.num_slices + 1)


def test_fusion_decisions_on_the_benchmark_tree():
    """No step is fused unless its options ask for it. Asked for everywhere
    (TSG_STEP_FUSE), the n=60 benchmark tree fuses its expansion steps in every ring: each
    fused producer is an operand of its consumer, launches nothing and needs no
    workspace, and the count rings' fused steps remove over 30% of their bytes; the
    global switch off restores the plain launches."""
    import json

    from tensorsat_gb300 import autotune

    plan = json.loads((HEADER.parent.parent / "plans" / "3sat_n60_m256_rng0_t26.json").read_text())
    cnf = CNFInstance.random(3, 60, 256, rng=0)
    c = GpuContraction.from_plan(CudaRel, cnf.clause_diagram().wiring, plan)
    npl = c.native_plan()
    lib = _native.lib()
    primes = PRIMES_31[:3]
    rings = (_native.TSG_RING_MODP, _native.TSG_RING_U64, _native.TSG_RING_OR_AND)
    assert lib.tsg_fusion_enabled() == 1
    assert npl.fused_steps(_native.TSG_RING_MODP, primes, 64, c.tree) == {}
    ws_plain = npl.workspace_bytes(_native.TSG_RING_MODP, 3, 64)
    n_plain = npl.launch_count(0, 64, 64, _native.TSG_RING_MODP, 3)
    try:
        for r in rings:
            autotune.fuse_all(c, r)
        fused = npl.fused_steps(_native.TSG_RING_MODP, primes, 64, c.tree)
        assert fused and fused == npl.fused_steps(_native.TSG_RING_U64, (), 64, c.tree)
        assert set(npl.fused_steps(_native.TSG_RING_OR_AND, (), 64, c.tree)) <= set(fused)
        L = c.tree.num_leaves
        for s, p in fused.items():
            assert L + p in c.tree.steps[s]
        assert npl.workspace_bytes(_native.TSG_RING_MODP, 3, 64) < ws_plain
        assert npl.launch_count(0, 64, 64, _native.TSG_RING_MODP, 3) == n_plain - len(fused)
        sp = c.sliced_plan
        saved = sp.bytes_per_slice(4, 3) - sp.bytes_per_slice(4, 3, fused)
        assert saved > 0.3 * sp.bytes_per_slice(4, 3)
        lib.tsg_set_fusion(0)
        assert npl.fused_steps(_native.TSG_RING_MODP, primes, 64, c.tree) == {}
        assert npl.workspace_bytes(_native.TSG_RING_MODP, 3, 64) == ws_plain
    finally:
        lib.tsg_set_fusion(1)
        for r in rings:
            autotune.set_options(c, r, None)
    assert n_plain == npl.launch_count(0, 64, 64)


def test_subset_dp_rejects_bad_sizes_and_nulls():
    lib = _native.lib()
    u64 = ctypes.c_uint64 * 4
    bits, keep, live = u64(1, 2, 4, 8), u64(0), u64(15)
    best = ctypes.c_double()
    split = (ctypes.c_uint32 * 16)()
    kept = (ctypes.c_uint64 * 16)()
    for n, words in [(0, 1), (21, 1), (4, 0), (4, 65)]:
        assert lib.tsg_plan_subset_dp(n, words, bits, keep, live, -1, ctypes.byref(best),
                                      split, kept) == _native.TSG_ERR_INVALID_ARGUMENT
    assert lib.tsg_plan_subset_dp(4, 1, None, keep, live, -1, ctypes.byref(best), split,
                                  kept) == _native.TSG_ERR_INVALID_ARGUMENT
    assert lib.tsg_plan_subset_dp(4, 1, bits, keep, live, -1, ctypes.byref(best), split,
                                  kept) == _native.TSG_OK
    # four disjoint one-wire inputs, nothing kept: no partial result keeps a wire, so each
    # of the 3 steps costs 2^0
    assert best.value == 3.0
    # every wire kept: pairs first, then the pair of pairs (4 + 4 + 16) beats a chain (28)
    assert lib.tsg_plan_subset_dp(4, 1, bits, u64(15), live, -1, ctypes.byref(best), split,
                                  kept) == _native.TSG_OK
    assert best.value == 24.0
    assert kept[15] == 15 and split[15] in (0b0011, 0b0101, 0b1001)


def test_wait_limit_setting_is_range_checked():
    """The bounded-wait limit of the streaming kernel is settable between 1 us and the 2 s
    default; values outside are rejected and leave the setting unchanged."""
    lib = _native.lib()
    default = lib.tsg_wait_limit_ns()
    assert default == 2_000_000_000
    try:
        assert lib.tsg_set_wait_limit_ns(999) == _native.TSG_ERR_INVALID_ARGUMENT
        assert lib.tsg_set_wait_limit_ns(3_000_000_000) == _native.TSG_ERR_INVALID_ARGUMENT
        assert lib.tsg_wait_limit_ns() == default
        assert lib.tsg_set_wait_limit_ns(1_000_000) == _native.TSG_OK
        assert lib.tsg_wait_limit_ns() == 1_000_000
    finally:
        assert lib.tsg_set_wait_limit_ns(default) == _native.TSG_OK
    assert lib.tsg_debug_stall_producer(-5) == _native.TSG_OK  # off


def test_step_options_change_kernel_choices_not_plans():
    """Per-step options (the autotuner's choices): TSG_STEP_NO_STREAM puts a streamed step
    on the tile kernel, TSG_STEP_NO_FUSE keeps a fused producer out of its consumer (its
    result is stored again, so the workspace grows); clearing restores the executor's
    choices. Unknown bits are rejected."""
    import json

    from tensorsat_gb300 import autotune

    plan = json.loads((HEADER.parent.parent / "plans" / "3sat_n60_m256_rng0_t26.json").read_text())
    cnf = CNFInstance.random(3, 60, 256, rng=0)
    c = GpuContraction.from_plan(CudaRel, cnf.clause_diagram().wiring, plan)
    npl = c.native_plan()
    ring, primes = _native.TSG_RING_MODP, PRIMES_31[:3]
    base = npl.describe(ring, primes, 64)
    ws = npl.workspace_bytes(ring, 3, 64)
    streamed = [s for s in range(npl.num_steps) if base[s][0] == _native.TSG_KERNEL_STREAM]
    assert streamed and npl.fused_steps(ring, primes, 64, c.tree) == {}
    try:
        autotune.fuse_all(c, ring)
        fused = npl.fused_steps(ring, primes, 64, c.tree)
        assert fused and npl.workspace_bytes(ring, 3, 64) < ws
        p = next(iter(fused.values()))
        opts = [_native.TSG_STEP_FUSE] * npl.num_steps
        opts[p] = _native.TSG_STEP_NO_FUSE
        unfused_stream = [s for s in streamed if s not in fused]
        opts[unfused_stream[0]] |= _native.TSG_STEP_NO_STREAM
        autotune.set_options(c, ring, opts)
        got = npl.describe(ring, primes, 64)
        assert got[unfused_stream[0]][0] == _native.TSG_KERNEL_TILE
        assert got[p][0] != _native.TSG_KERNEL_NONE
        # other rings keep their own (empty) options: nothing fused there
        assert npl.fused_steps(_native.TSG_RING_U64, (), 64, c.tree) == {}
        npl.validate(ring, primes, 0, 128, 64)
        bad = list(opts)
        bad[0] = 16
        with pytest.raises(_native.TsgValueError):
            autotune.set_options(c, ring, bad)
    finally:
        autotune.set_options(c, ring, None)
    assert (npl.describe(ring, primes, 64) == base).all()
    assert npl.workspace_bytes(ring, 3, 64) == ws


def test_tuning_cache_round_trip(tmp_path):
    """A cached tuning entry is found under its plan, ring, moduli and GPU name, and
    applying it sets its options and returns its group."""
    import json

    from tensorsat_gb300 import autotune

    cnf = CNFInstance.random(3, 30, 128, rng=0)
    c = _plan_for(cnf, 14)
    npl = c.native_plan()
    ring, primes = _native.TSG_RING_MODP, PRIMES_31[:3]
    opts = [_native.TSG_STEP_NO_STREAM] * npl.num_steps
    entry = {"ring": ring, "primes": list(primes), "group": 4, "options": opts}
    path = tmp_path / "plan.tune.json"
    path.write_text(json.dumps({"format": autotune.TUNE_FORMAT, "entries": {
        autotune.entry_key(c, ring, primes, "GB300 test"): entry}}))
    assert autotune.load(path, c, ring, primes, gpu="other GPU") is None
    assert autotune.load(path, c, _native.TSG_RING_U64, (), gpu="GB300 test") is None
    got = autotune.load(path, c, ring, primes, gpu="GB300 test")
    assert got == entry
    try:
        assert autotune.apply(c, got) == 4
        kinds = npl.describe(ring, primes, 4)
        assert all(k[0] != _native.TSG_KERNEL_STREAM for k in kinds)
    finally:
        autotune.set_options(c, ring, None)
    (tmp_path / "bad.json").write_text('{"format": "x"}')
    with pytest.raises(ValueError):
        autotune.load(tmp_path / "bad.json", c, ring, primes, gpu="GB300 test")


def test_variant_runs_size_their_workspace_per_slot():
    """A variant run lays out every step per slot (variant x slice): its workspace grows
    with the variants and is at least that of a plain run of the same slices; counts and
    strides that are not powers of two are rejected before any device work."""
    c = _plan_for(CNFInstance.random(3, 20, 85, rng=2), 8)
    npl = c.native_plan()
    lib = _native.lib()
    out = ctypes.c_int64()
    ring = _native.TSG_RING_MODP
    sizes = []
    for nv in (1, 2, 8):
        _native.check(lib.tsg_plan_variants_workspace_bytes(npl.handle, ring, 3, 2, nv,
                                                            ctypes.byref(out)))
        sizes.append(out.value)
    assert sizes[0] >= npl.workspace_bytes(ring, 3, 2)
    assert sizes[0] < sizes[1] < sizes[2]
    assert lib.tsg_plan_variants_workspace_bytes(npl.handle, ring, 3, 2, 3,
                                                 ctypes.byref(out)) == _native.TSG_ERR_INVALID_ARGUMENT
    p = (ctypes.c_uint32 * 3)(*PRIMES_31[:3])
    for nv, stride in ((3, 1 << 12), (2, 1000), (2, 8)):
        assert lib.tsg_plan_run_variants(npl.handle, ring, 3, p, 16, stride, nv, 2, 256, 1 << 20,
                                         16, 0, None) == _native.TSG_ERR_INVALID_ARGUMENT
