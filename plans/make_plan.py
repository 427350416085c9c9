"""Makes the learned-path plan of the n=60 benchmark instance (3-SAT, n=60, m=256, seed 0):
the committed cost model (plans/costmodel_n60.npz) ranks the planner's candidate trees for
the instance's clause network by predicted device time, and the candidate it ranks first
is written as a plan file (format tensorsat_gb300.plan/1, with a "chosen_by" record of the
ranking). The planner's own tree is candidate 0, so the learned path falls back to it
whenever the model ranks it first. With --measure K, the K best-ranked candidates and the
planner's tree are also timed on the GPU (device milliseconds per slice over 16 slices,
3-prime count + OR-AND), for the record; the choice stays the model's.

    python plans/make_plan.py [--candidates 64] [--measure 4]

Needs a GPU (the model's layers run on the tensor cores). The autotuner entry of the new
plan is made afterwards by `python bench.py --tree learned --tune`.
"""

from __future__ import annotations

import argparse
import json
import math
import multiprocessing as mp
import os
import sys
import time
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

OUT = HERE / "3sat_n60_m256_rng0_learned.json"
MODEL = HERE / "costmodel_n60.npz"
GROUP = 16  # slices per measured group, as in the model's training data


def main() -> None:
    p = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    p.add_argument("--candidates", type=int, default=64)
    p.add_argument("--measure", type=int, default=4,
                   help="time the K best-ranked candidates and the planner's tree")
    p.add_argument("--out", default=str(OUT))
    args = p.parse_args()

    from tensorsat_gb300 import _native, costmodel
    from tensorsat_gb300.lib.sat import CNFInstance

    _native.lib()  # built (if needed) once here, not in every worker
    cnf = CNFInstance.random(3, 60, 256, rng=0)
    t0 = time.perf_counter()
    with mp.get_context("spawn").Pool(os.cpu_count() or 1) as pool:
        cands = costmodel.cnf_candidates(pool, [cnf], args.candidates)[0]
    plan_s = time.perf_counter() - t0

    import numpy as np
    import torch

    from tensorsat_gb300.contractions.gpu import PRIMES_31, GpuContraction
    from tensorsat_gb300.lang.cuda_rel import CudaRel

    torch.cuda.set_device(0)
    primes = PRIMES_31[:3]
    diagram = cnf.clause_diagram()
    cons = [GpuContraction(CudaRel, diagram.wiring, tree=t, sliced=s) for t, s in cands]
    model = costmodel.CostModel(seed=0)
    model.load_state(dict(np.load(MODEL)))
    pred = costmodel.rank(model, cons, GROUP, primes)  # predicted device ms per instance
    order = sorted(range(len(cons)), key=lambda j: pred[j])
    pick = order[0]
    measured = {}
    for j in sorted(set(order[:args.measure]) | {0}) if args.measure > 0 else []:
        measured[j] = costmodel.measure(cons[j], diagram, primes, GROUP, passes=2) * \
            cons[j].num_slices
    plan = cons[pick].plan_dict()
    plan["chosen_by"] = {
        "rule": "committed cost model's lowest predicted device time among the planner's "
                "candidate trees of the instance (candidate 0: the planner's usual choice)",
        "instance": "CNFInstance.random(3, 60, 256, rng=0), clause network",
        "candidates": len(cons), "picked": pick,
        "predicted_ms_per_instance": {str(j): round(pred[j], 1) for j in order[:8] + [0]},
        "measured_ms_per_instance": {str(j): round(v, 1) for j, v in measured.items()},
        "slices": {str(j): cons[j].num_slices for j in order[:8] + [0]},
        "planning_s": round(plan_s, 1),
    }
    Path(args.out).write_text(json.dumps(plan, separators=(",", ":")) + "\n")
    print(json.dumps(plan["chosen_by"]), flush=True)
    if measured and 0 in measured and pick in measured:
        print(f"planner tree {measured[0]:.0f} ms, learned tree {measured[pick]:.0f} ms: "
              f"{measured[0] / measured[pick]:.2f}x", flush=True)
    if not all(math.isfinite(v) for v in pred):
        raise RuntimeError("non-finite predictions")


if __name__ == "__main__":
    main()
