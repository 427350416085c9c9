"""The streaming kernel's bounded waits run out, report TSG_ERR_TIMEOUT and leave the
device usable.

Every mbarrier wait of the streaming kernel gives up after a limit (2 s by default). This
test makes one run out on purpose without any fault: it shortens the limit to 1 ms and
makes every producer warp stop after its first stage (tsg_debug_stall_producer). The
producer then issues no further copy and arms no further barrier, so no copy is in flight
when the consumers give up; each consumer warp waits 1 ms for the next stage, records
TSG_ERR_TIMEOUT and returns, and the producer waits for its one stage's copies before its
block exits. The host reads the record once (TSG_ERR_TIMEOUT), a second read is clean,
and a normal run on the same stream afterwards gives the exact model count.
"""

from __future__ import annotations

import pytest

from oracle import finrel_oracle as orc
from tensorsat_gb300 import _device, _native
from tensorsat_gb300.contractions.gpu import PRIMES_31, GpuContraction
from tensorsat_gb300.lang.cuda_rel import CudaRel
from tensorsat_gb300.lib.sat import CNFInstance

pytestmark = pytest.mark.gpu


def test_stalled_producer_times_out_and_the_next_run_is_exact(cuda):
    lib = _native.lib()
    cnf = CNFInstance.random(3, 44, 187, rng=1)
    d = cnf.clause_diagram()
    c = GpuContraction(CudaRel, d.wiring, target_bits=22, trials=2, seed=0)
    primes = PRIMES_31[:3]
    # fused steps off for this plan's layouts, so that its largest step streams
    fusion = lib.tsg_fusion_enabled()
    lib.tsg_set_fusion(0)
    kinds = c.native_plan().describe(_native.TSG_RING_MODP, primes, 4)
    assert any(k[0] == _native.TSG_KERNEL_STREAM for k in kinds), "no streamed step"
    stream = _device.stream_handle()
    assert lib.tsg_take_device_error(stream) == _native.TSG_OK  # clean start
    default = lib.tsg_wait_limit_ns()
    try:
        _native.check(lib.tsg_set_wait_limit_ns(1_000_000))
        _native.check(lib.tsg_debug_stall_producer(1))
        c.run(d, _native.TSG_RING_MODP, primes, slice_range=(0, 4), group=4)
        assert lib.tsg_take_device_error(stream) == _native.TSG_ERR_TIMEOUT
        assert "bounded device-side wait" in lib.tsg_last_error().decode()
        assert lib.tsg_take_device_error(stream) == _native.TSG_OK  # the record was cleared
    finally:
        lib.tsg_debug_stall_producer(-1)
        lib.tsg_set_wait_limit_ns(default)
        lib.tsg_set_fusion(fusion)
    expected = orc.dpll_count(cnf.num_vars, cnf.clauses)[0]
    assert c.count(d, ring="modp", num_primes=3, group=4) == expected
    assert c.count(d, ring="u64", group=4) == expected
    assert bool(c.contract(d, group=4)) == (expected > 0)
