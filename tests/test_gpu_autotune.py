"""The autotuner on the GPU: it times the executor's kernel choices against unfused,
tile-only and fully fused configurations and a per-decision mix, keeps the fastest per
slice, caches the choice, and the tuned plan gives the exact answer."""

from __future__ import annotations

import pytest

from oracle import finrel_oracle as orc
from tensorsat_gb300 import _native, autotune
from tensorsat_gb300.contractions.gpu import PRIMES_31, GpuContraction
from tensorsat_gb300.lang.cuda_rel import CudaRel
from tensorsat_gb300.lib.sat import CNFInstance

pytestmark = pytest.mark.gpu


def test_tuned_plan_is_cached_and_exact(cuda, tmp_path):
    cnf = CNFInstance.random(3, 44, 187, rng=1)
    d = cnf.clause_diagram()
    c = GpuContraction(CudaRel, d.wiring, target_bits=22, trials=2, seed=0)
    ring, primes = _native.TSG_RING_MODP, PRIMES_31[:3]
    path = tmp_path / "plan.tune.json"
    try:
        entry = autotune.load_or_tune(path, c, d, ring, primes, budget_bytes=4 << 30)
        assert {t["config"] for t in entry["trials"]} == {"executor", "no_fuse", "tile",
                                                          "fuse", "plane_split", "mixed"}
        assert entry["ms_per_slice"] <= entry["default_ms_per_slice"]
        assert len(entry["options"]) == c.native_plan().num_steps
        assert autotune.load_or_tune(path, c, d, ring, primes) == entry  # from the cache
        want = orc.dpll_count(cnf.num_vars, cnf.clauses)[0]
        assert c.count(d, ring="modp", num_primes=3, group=entry["group"]) == want
    finally:
        autotune.set_options(c, ring, None)
