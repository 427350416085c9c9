"""The allocation-free tree-executor entry point (tsg_plan_run_static).

Some callers cannot allocate device memory: host bindings that only hand over pointers to
buffers the application already owns, or services that must not grow their device memory
after start-up. tsg_plan_run_static serves them with a library-owned 64 MiB scratch array
instead of a caller workspace. These tests call it through the C ABI and require exactly
the results of tsg_plan_run (counts and SAT bits are integers: equality is the tolerance)
on two calls in a row, since every call reuses the same array.

This file is collected last so that a run stopping at its first failure has run every
other test before it; it also passes on its own in a fresh process.
"""

from __future__ import annotations

import ctypes

import numpy as np
import pytest
import torch

from oracle import finrel_oracle as orc
from tensorsat_gb300 import _device, _native
from tensorsat_gb300.contractions.gpu import PRIMES_31, GpuContraction
from tensorsat_gb300.lang.cuda_rel import CudaRel
from tensorsat_gb300.lib.sat import CNFInstance

pytestmark = pytest.mark.gpu


def _run_static(npl, ring, primes, pool, ns, group, result):
    lib = _native.lib()
    parr = (ctypes.c_uint32 * max(1, len(primes)))(*primes)
    st = lib.tsg_plan_run_static(npl.handle, ring, len(primes), parr, pool.data_ptr(), 0, ns,
                                 group, result.data_ptr(), 0, _device.stream_handle())
    _native.check(st)


@pytest.mark.parametrize("ring,primes", [(_native.TSG_RING_MODP, PRIMES_31[:3]),
                                         (_native.TSG_RING_U64, ()),
                                         (_native.TSG_RING_OR_AND, ())])
def test_static_scratch_matches_workspace_entry_point(cuda, ring, primes):
    cnf = CNFInstance.random(3, 20, 85, rng=2)
    d = cnf.clause_diagram()
    c = GpuContraction(CudaRel, d.wiring, target_bits=8, trials=1)
    npl = c.native_plan()
    ns = c.num_slices
    group = min(8, ns)
    assert npl.workspace_bytes(ring, max(1, len(primes)), group) <= \
        _native.lib().tsg_static_scratch_bytes()
    pool = c.leaf_pool(d)
    for _ in range(2):  # the array keeps the previous call's contents
        expected = c.run(None, ring, primes=primes, pool=pool, group=group)
        got = torch.zeros_like(expected)
        _run_static(npl, ring, primes, pool, ns, group, got)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(got.cpu().numpy(), expected.cpu().numpy())
    count = orc.brute_force_count(20, cnf.clauses)
    if ring == _native.TSG_RING_U64:
        assert int(got.cpu().numpy().view(np.uint64)[0]) * c.discard_factor == count
    elif ring == _native.TSG_RING_OR_AND:
        assert int(got.cpu().numpy()[0]) == int(count > 0)


def test_static_scratch_rejects_plans_above_its_size(cuda):
    cnf = CNFInstance.random(3, 40, 170, rng=0)
    d = cnf.clause_diagram()
    c = GpuContraction(CudaRel, d.wiring, target_bits=22, trials=1)
    npl = c.native_plan()
    group = min(c.num_slices, 64)
    limit = _native.lib().tsg_static_scratch_bytes()
    assert npl.workspace_bytes(_native.TSG_RING_MODP, 3, group) > limit
    pool = c.leaf_pool(d)
    res = torch.zeros(3, dtype=torch.int32, device=cuda)
    with pytest.raises(_native.TsgError) as err:
        _run_static(npl, _native.TSG_RING_MODP, PRIMES_31[:3], pool, c.num_slices, group, res)
    assert err.value.status == _native.TSG_ERR_WORKSPACE
    assert "64 MiB" in str(err.value)
