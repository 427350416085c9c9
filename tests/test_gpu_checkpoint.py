"""The checkpointed sliced count on the GPU: chunks of slices counted by the device, the
file records each finished chunk, an interrupted run resumes with the chunks still missing,
and the total equals the one-call count and the oracle's brute-force count (integers:
equality)."""

from __future__ import annotations

import json

import pytest

from oracle import finrel_oracle as orc
from tensorsat_gb300.contractions.gpu import GpuContraction
from tensorsat_gb300.lang.cuda_rel import CudaRel
from tensorsat_gb300.lib.sat import CNFInstance

pytestmark = pytest.mark.gpu


def test_checkpointed_count_on_the_device_resumes(cuda, tmp_path, monkeypatch):
    cnf = CNFInstance.random(3, 22, 80, rng=11)
    d = cnf.clause_diagram()
    want = orc.brute_force_count(cnf.num_vars, cnf.clauses)
    assert want > 0
    c = GpuContraction(CudaRel, d.wiring, target_bits=8, trials=1)
    ns = c.num_slices
    assert ns >= 16
    assert c.count(d, ring="modp", num_primes=2) == want
    real = GpuContraction.count
    calls = []

    def interrupted(self, diagram, **kw):
        calls.append(kw["slice_range"])
        if len(calls) == 4:
            raise RuntimeError("interrupted")
        return real(self, diagram, **kw)

    path = tmp_path / "count.json"
    monkeypatch.setattr(GpuContraction, "count", interrupted)
    with pytest.raises(RuntimeError):
        c.count_checkpointed(d, path, chunk_slices=ns // 8, group=2)
    monkeypatch.setattr(GpuContraction, "count", real)
    done = json.loads(path.read_text())
    assert len(done["done"]) == 3
    assert c.count_checkpointed(d, path, chunk_slices=ns // 8, group=2) == want
    assert len(json.loads(path.read_text())["done"]) == 8
