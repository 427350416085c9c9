"""The large sliced 5-SAT pipeline on the GPU: uniform random 5-SAT at clause ratio 21, the
tree sliced over 8 wires (256 slices), the OR-AND decision contraction and the 3-prime
modular count run as batched slice launches combined on the device.

The configuration as written (n=100, m=2100, at most 2^30 entries per intermediate) admits
no tree at all (``test_planner.py`` gives the bound), so the pipeline runs
* at a brute-force size (n=24, m=504), and
* at the largest n whose tree meets the 2^30 cap with 8 sliced wires (n=39, m=819), where
  the exact DPLL counter of the oracle pins the count (brute force would take hours).
Integers throughout: the tolerance is equality.
"""

from __future__ import annotations

import time

import pytest
import torch

from oracle import finrel_oracle as orc
from tensorsat_gb300.contractions.gpu import GpuContraction
from tensorsat_gb300.lang.cuda_rel import CudaRel
from tensorsat_gb300.lib.sat import CNFInstance

pytestmark = pytest.mark.gpu


def test_5sat_n24_256_slices_match_brute_force(cuda):
    cnf = CNFInstance.random(5, 24, 504, rng=0)
    d = cnf.clause_diagram()
    c = GpuContraction(CudaRel, d.wiring, target_bits=15, trials=2)
    assert c.num_slices == 256
    exp = orc.brute_force_count(24, cnf.clauses)
    assert c.count(d, ring="modp", num_primes=3, group=64) == exp
    assert c.count(d, ring="u64", group=256) == exp
    assert bool(c.contract(d, group=16)) == (exp > 0)


def test_5sat_n39_2_30_cap_256_slices_match_dpll(cuda):
    cnf = CNFInstance.random(5, 39, 819, rng=0)
    d = cnf.clause_diagram()
    c = GpuContraction(CudaRel, d.wiring, target_bits=30, trials=2)
    assert c.num_slices == 256 and c.stats()["peak_bits"] == 30
    exp, _ = orc.dpll_count(39, cnf.clauses)
    try:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        got = c.count(d, ring="modp", num_primes=3, group=2)  # about 70 GiB of workspace
        t1 = time.perf_counter()
        sat = bool(c.contract(d, group=4))
        t2 = time.perf_counter()
        print(f"5-SAT n=39 m=819, 256 slices of 2^30: 3-prime count {t1 - t0:.2f} s, "
              f"SAT bit {t2 - t1:.2f} s")
    finally:
        torch.cuda.empty_cache()
    assert got == exp
    assert sat == (exp > 0)
