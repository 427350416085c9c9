"""Benchmark: exact model count + SAT bit of uniform random 3-SAT, n=60, m=256, on GB300.

Workload (the single-instance #SAT configuration): ``CNFInstance.random(3, 60, 256,
rng=SEED)`` compiled to its clause network (one 2x2x2 {0,1} tensor per clause), one
contraction tree from the project's planner with every intermediate capped at 2^26 entries
by slicing. The exact count is carried modulo three 31-bit primes (uint32 residue planes,
CRT on the host); the SAT bit is the OR-AND contraction of the same tree.

A *step* contracts G slices of that instance in both rings (count and SAT
bit). Every slice of an instance runs the same kernels on the same shapes, so
``instances/s = slices/s / slices per instance`` is exact for this instance. Inputs
(leaves) are resident in HBM for ``value``; ``e2e`` goes through the public API
(``GpuContraction.count`` / ``.contract``) from host leaves to host results each step.

The tree is the committed plan ``plans/3sat_n60_m256_rng0_t26.json`` (the project's
planner with ``target_bits=26, trials=8, seed=0``; ``--replan`` plans again), so both arms
contract the same tree and the reference arm loads no native code.

The autotuner's committed entries for that plan and GPU (``plans/*.tune.json``) set the
slice group per ring and the per-step kernel options (``--no-tuning`` runs the executor's
own choices).

``batched`` (default run, one GPU): a bounded ragged batch of random 3-SAT instances (n
uniform in [30, 40], clause ratio uniform in [3.5, 5.0], seeded per instance), planned on
the host cores before the first CUDA call, timed as captured-graph replays (small steps of
a tree level packed across instances, and one launch per step for comparison), in the
plain per-instance form (``GpuContraction.count`` + ``.contract``) and in the serving forms
(``BatchContraction.serve`` pipelined over a stream of input batches; ``load`` +
``graph=True`` one call after the other), with every count and SAT bit checked against the
oracle's DPLL counts.

``learned`` (default run): the committed cost model ranks 64 planner candidates of each of
8 held-out n=60 instances; its picks and the planner's trees are timed on the device.

Other workloads: ``--workload ragged`` (the batch alone), ``costmodel`` (train and
evaluate the cost model), ``costmodel-eval`` (evaluate the committed weights on held-out
instances), ``costmodel-gemm`` (the cost model's tensor-core layer against cuBLAS).

``--impl reference`` times the reference's CPU path for the same workload (the oracle's
restatement of the upstream numpy contraction: per-slice einsum in the OR-AND semiring and
over exact integers), one slice per process on all host cores.

Prints one JSON line (rank 0).
"""

from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "exact instances/s (SAT bit + model count), uniform random 3-SAT n=60 m=256"
UNIT = "instances/s"
N_VARS, N_CLAUSES = 60, 256
TARGET_BITS = 26
NUM_PRIMES = 3
# committed plans of the headline instance: the planner's tree (8 trials, with its
# autotuner entries) and the learned path's tree (the committed cost model's pick among 64
# planner candidates, plans/make_plan.py; tuned on demand with --tree learned --tune)
PLAN_FILES = {"planner": ROOT / "plans" / "3sat_n60_m256_rng0_t26.json",
              "learned": ROOT / "plans" / "3sat_n60_m256_rng0_learned.json"}
TUNE_FILES = {k: v.with_name(v.stem + ".tune.json") for k, v in PLAN_FILES.items()}


def parse_args():
    p = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--seed", type=int, default=0)
    p.add_argument("--group", type=int, default=0, help="slices per step (0 = auto)")
    p.add_argument("--trials", type=int, default=8)
    p.add_argument("--e2e-steps", type=int, default=3)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--learned-instances", type=int, default=8,
                   help="held-out n=60 instances of the learned-path leg of the default run")
    p.add_argument("--learned-candidates", type=int, default=64,
                   help="planner candidate trees the cost model ranks per instance")
    p.add_argument("--cm-train", type=int, default=320, help="costmodel: training instances")
    p.add_argument("--cm-heldout", type=int, default=64, help="costmodel: held-out n=60 instances")
    p.add_argument("--cm-epochs", type=int, default=150, help="costmodel: training epochs")
    p.add_argument("--cm-out", default="", help="costmodel: write the trained weights (.npz)")
    p.add_argument("--workload", default="n60",
                   choices=["n60", "ragged", "costmodel", "costmodel-eval", "costmodel-gemm"],
                   help="n60: the single-instance headline workload; ragged: a batch of "
                        "random instances of uneven sizes (batched runs, CUDA graphs)")
    p.add_argument("--instances", type=int, default=512, help="ragged: batch size")
    p.add_argument("--n-range", type=int, nargs=2, default=[30, 40], help="ragged: n bounds")
    p.add_argument("--plan-only", action="store_true",
                   help="ragged: plan the batch on the host cores and print its algorithmic "
                        "bytes per n (no GPU, no timing of contractions)")
    p.add_argument("--replan", action="store_true",
                   help="plan the n=60 tree instead of loading the committed plan")
    p.add_argument("--no-batched", action="store_true",
                   help="skip the ragged batched-vs-plain leg of the default run")
    p.add_argument("--tune", action="store_true",
                   help="run the autotuner for the n=60 plan when its tuning file has no "
                        "entry for this GPU, and store the entry")
    p.add_argument("--tree", choices=["learned", "planner"], default=None,
                   help="committed n=60 tree: the planner's own (default) or the learned "
                        "path's pick")
    p.add_argument("--tune-file", default=None,
                   help="tuning file of the n=60 plan (read, and written by --tune; default: "
                        "the one beside the chosen plan)")
    p.add_argument("--no-tuning", action="store_true",
                   help="ignore the committed tuning (the executor's own kernel choices)")
    p.add_argument("--no-instance", action="store_true",
                   help="skip the whole-instance count and its DPLL check")
    p.add_argument("--batched-steps", type=int, default=3,
                   help="timed graph-replay passes of the ragged leg")
    return p.parse_args()


def measured_peaks() -> tuple[float, str]:
    path = ROOT / "MEASURED_PEAKS.json"
    try:
        data = json.loads(path.read_text())
        return float(data["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int) -> None:
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.thread.join(timeout=5)

    def summary(self) -> dict:
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for name, val in zip(names, parts[3:7]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


def tree_choice(args) -> str:
    """The committed n=60 tree to run: the planner's (default) or the learned path's pick.
    On this instance the current weights rank a candidate first that measures 0.90x the
    planner's tree (recorded in the learned plan file), so the headline runs the planner's
    tree; the learned path's gain is measured on held-out instances (the learned leg)."""
    return args.tree if args.tree is not None else "planner"


def committed_plan(args) -> dict | None:
    """The committed plan of the headline workload (seed 0, 8 trials), unless replanning."""
    path = PLAN_FILES[tree_choice(args)]
    if args.replan or args.seed != 0 or args.trials != 8 or not path.exists():
        return None
    return json.loads(path.read_text())


def build_workload(args):
    from tensorsat_gb300.contractions.gpu import GpuContraction
    from tensorsat_gb300.lang.cuda_rel import CudaRel
    from tensorsat_gb300.lib.sat import CNFInstance

    cnf = CNFInstance.random(3, N_VARS, N_CLAUSES, rng=args.seed)
    diagram = cnf.clause_diagram()
    plan = committed_plan(args)
    if plan is not None:
        contraction = GpuContraction.from_plan(CudaRel, diagram.wiring, plan)
    else:
        contraction = GpuContraction(CudaRel, diagram.wiring, target_bits=TARGET_BITS,
                                     trials=args.trials, seed=0)
    return cnf, diagram, contraction


class PlanView:
    """The tree facts the CPU arm and the config need (steps, sliced wires, slice count,
    cost), read from a plan without building a GPU contraction."""

    def __init__(self, tree, sliced) -> None:
        self.tree = tree
        self.sliced_wires = tuple(sliced)
        self.num_slices = 1 << len(self.sliced_wires)

    def stats(self) -> dict:
        tot, peak, _ = self.tree.cost(frozenset(self.sliced_wires))
        return {"num_sliced": len(self.sliced_wires), "log2_index_space_per_slice": tot,
                "peak_bits": peak}


def reference_workload(args):
    """Instance and tree of the CPU arm: the committed plan when it applies (no native
    code is loaded), else the planner."""
    from tensorsat_gb300 import planner
    from tensorsat_gb300.lib.sat import CNFInstance

    cnf = CNFInstance.random(3, N_VARS, N_CLAUSES, rng=args.seed)
    plan = committed_plan(args)
    if plan is not None:
        tree, sliced = planner.plan_from_dict(plan)
        return cnf, PlanView(tree, sliced)
    _, _, contraction = build_workload(args)
    return cnf, PlanView(contraction.tree, contraction.sliced_wires)


# --------------------------------------------------------------------------------------
# CPU leg (oracle port of the reference's numpy path), one slice per process


def _cpu_slice(args):
    clauses, steps, sliced, sid = args
    from oracle import finrel_oracle as orc

    fixed = {w: (sid >> j) & 1 for j, w in enumerate(sliced)}
    count = orc.cnf_count_by_tree(N_VARS, clauses, steps, "count", fixed=fixed)
    sat = orc.cnf_count_by_tree(N_VARS, clauses, steps, "or_and", fixed=fixed)
    return count, sat


def cpu_pool(cores: int):
    import multiprocessing as mp

    return mp.get_context("spawn").Pool(cores)


def cpu_sample(pool, cores: int, cnf, contraction, first_slice: int):
    steps = list(contraction.tree.steps)
    sliced = list(contraction.sliced_wires)
    ns = contraction.num_slices
    jobs = [(cnf.clauses, steps, sliced, (first_slice + i) % ns) for i in range(cores)]
    t0 = time.perf_counter()
    results = pool.map(_cpu_slice, jobs)
    dt = time.perf_counter() - t0
    return dt, results


def run_reference(args) -> None:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    pool = cpu_pool(cores)
    cnf, contraction = reference_workload(args)
    ns = contraction.num_slices
    for w in range(args.warmup):
        cpu_sample(pool, cores, cnf, contraction, w * cores)
    times = []
    for k in range(args.steps):
        dt, _ = cpu_sample(pool, cores, cnf, contraction, (args.warmup + k) * cores)
        times.append(dt)
    pool.close()
    total = sum(times)
    value = args.steps * cores / ns / total
    sample = (f"{cores} slices of {ns} per step (one per process), count over exact "
              f"integers + OR-AND bit per slice")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000 * total / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "uint64/uint8 (numpy einsum)",
        "data": "synthetic (seeded CNFInstance.random)",
        "config": workload_config(args, contraction, group=cores),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


DRAM_PROFILES = {"planner": ROOT / "profiles" / "tree_steps_n60_dram.txt",
                 "learned": ROOT / "profiles" / "tree_steps_n60_learned_dram.txt"}


def dominant_traffic(ring: str, step: int, group: int, plan_sha: str):
    """DRAM bytes (read + write) of one launch of tree step `step` in `ring`, from the ncu
    launch list committed under profiles/ for this plan (the file whose "# plan <sha256>"
    line names it), or None when no capture of this plan holds this step at this group
    size."""
    text = next((p.read_text() for p in DRAM_PROFILES.values()
                 if p.exists() and f"# plan {plan_sha}" in p.read_text()), None)
    if text is None:
        return None
    for line in text.splitlines():
        parts = line.split("#")[0].split()
        if len(parts) == 5 and parts[0] == ring and parts[1] == str(step) and parts[2] == str(group):
            try:
                return float(parts[4])
            except ValueError:
                return None
    return None


def tree_text(args) -> str:
    plan = committed_plan(args)
    if plan is None:
        return "replanned by the planner"
    if tree_choice(args) == "planner":
        return "the planner's tree, 8 trials (plans/3sat_n60_m256_rng0_t26.json)"
    cb = plan.get("chosen_by", {})
    picked = cb.get("picked")
    return (f"learned path: the committed cost model's pick among {cb.get('candidates')} planner "
            f"candidates (plans/3sat_n60_m256_rng0_learned.json): candidate {picked}"
            + (", the planner's own tree" if picked == 0 else ""))


def workload_config(args, contraction, group: int) -> dict:
    st = contraction.stats()
    return {
        "workload": f"3-SAT n={N_VARS} m={N_CLAUSES} rng={args.seed}, clause network, "
                    f"peak 2^{TARGET_BITS} entries",
        "k": 3, "n": N_VARS, "m": N_CLAUSES, "seed": args.seed,
        "slices_per_instance": contraction.num_slices,
        "sliced_wires": st["num_sliced"],
        "log2_index_space_per_slice": round(st["log2_index_space_per_slice"], 3),
        "slices_per_step": group,
        "tree": tree_text(args),
        "count_ring": f"mod {NUM_PRIMES} primes < 2^31 (CRT)",
        "l2": "inputs larger than L2 (intermediates up to 2^26 entries x slices)",
    }


# --------------------------------------------------------------------------------------
# GPU leg


def run_gb300(args) -> None:
    import torch

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    cores = os.cpu_count() or 1
    want_cpu = rank == 0 and world == 1 and not args.no_cpu_baseline
    want_batched = rank == 0 and world == 1 and not args.no_batched

    from tensorsat_gb300 import _native
    from tensorsat_gb300.contractions.gpu import PRIMES_31

    lib = _native.lib()  # builds the library if needed, before the workers load it
    # host work before the first CUDA call: spawned workers, the ragged batch's plans and
    # DPLL counts
    pool = cpu_pool(cores) if (want_cpu or want_batched) else None
    ragged = None
    if want_batched:
        lo, hi = args.n_range
        ragged = ragged_prepare(pool, args.instances, lo, hi)
    learned_prep = None
    if want_batched and args.learned_instances > 0:
        held = costmodel_heldout(args.learned_instances)
        cands = candidates_parallel(pool, held, args.learned_candidates)
        dpll_held = pool.map(_dpll_instance, [(c.num_vars, c.clauses) for c in held])
        learned_prep = (held, cands, dpll_held)
    cnf, diagram, contraction = build_workload(args)
    # the checker's exact count of the whole instance (DPLL, in a spawned worker)
    dpll = pool.apply_async(_dpll_instance, ((cnf.num_vars, cnf.clauses),)) if pool else None
    npl = contraction.native_plan()
    primes = PRIMES_31[:NUM_PRIMES]
    ns = contraction.num_slices
    dev = torch.device("cuda", local)
    # the autotuner's per-step kernel choices (committed beside the plan, measured on this
    # GPU model); --tune measures and stores them when missing
    tuning = None
    if committed_plan(args) is not None and not args.no_tuning:
        from tensorsat_gb300 import autotune

        tune_file = Path(args.tune_file or TUNE_FILES[tree_choice(args)])
        entries = {r: autotune.load(tune_file, contraction, r, p)
                   for r, p in ((_native.TSG_RING_MODP, primes), (_native.TSG_RING_OR_AND, ()))}
        if args.tune and any(e is None for e in entries.values()):
            free, _ = torch.cuda.mem_get_info()
            for r, p in ((_native.TSG_RING_MODP, primes), (_native.TSG_RING_OR_AND, ())):
                entries[r] = autotune.load_or_tune(tune_file, contraction, diagram, r, p,
                                                   budget_bytes=int(free * 0.4))
        if all(e is not None for e in entries.values()):
            for e in entries.values():
                autotune.apply(contraction, e)
            tuning = {("modp" if r == _native.TSG_RING_MODP else "or_and"):
                      {"group": e["group"], "config": e["config"], "gain": round(e["gain"], 4),
                       "steps_changed": sum(1 for o in e["options"] if o)}
                      for r, e in entries.items()}
    # slice groups: one per ring (the tuned ones when a tuning applies), and a step covers
    # `group` slices (the larger of the two) in both rings
    free, _ = torch.cuda.mem_get_info()
    budget = int(free * 0.75)

    def fits(gm: int, go: int) -> bool:
        return (npl.workspace_bytes(_native.TSG_RING_MODP, NUM_PRIMES, gm)
                + npl.workspace_bytes(_native.TSG_RING_OR_AND, 1, go)) <= budget

    if args.group:
        g_modp = g_or = args.group
    elif tuning is not None:
        g_modp = min(ns, tuning["modp"]["group"])
        g_or = min(ns, tuning["or_and"]["group"])
        while g_or > g_modp and not fits(g_modp, g_or):
            g_or //= 2
    else:
        g_modp = min(ns, 256)
        while g_modp > 1 and not fits(g_modp, g_modp):
            g_modp //= 2
        g_or = g_modp
    group = max(g_modp, g_or)
    ws_count = torch.empty(npl.workspace_bytes(_native.TSG_RING_MODP, NUM_PRIMES, g_modp),
                           dtype=torch.uint8, device=dev)
    ws_sat = torch.empty(npl.workspace_bytes(_native.TSG_RING_OR_AND, 1, g_or),
                         dtype=torch.uint8, device=dev)
    pool_dev = contraction.leaf_pool(diagram)
    res_count = torch.zeros(NUM_PRIMES, dtype=torch.int32, device=dev)
    res_sat = torch.zeros(1, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)
    sh = int(stream.cuda_stream)
    groups_per_instance = ns // group

    def slice_range(i: int) -> tuple[int, int]:
        g = (rank * (args.warmup + args.steps) + i) % groups_per_instance
        return g * group, (g + 1) * group

    def step(i: int) -> None:
        b, e = slice_range(i)
        npl.run(_native.TSG_RING_MODP, primes, pool_dev, b, e, g_modp, ws_count, res_count,
                False, sh)
        npl.run(_native.TSG_RING_OR_AND, (), pool_dev, b, e, g_or, ws_sat, res_sat, False, sh)

    for i in range(args.warmup):
        step(i)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    with ClockSampler(local) as clocks:
        ev[0].record(stream)
        for k in range(args.steps):
            step(args.warmup + k)
            ev[k + 1].record(stream)
        torch.cuda.synchronize()
    if dist:
        dist.barrier()
    step_ms = [ev[k].elapsed_time(ev[k + 1]) for k in range(args.steps)]
    elapsed = sum(step_ms) / 1000.0
    if dist:
        t = torch.tensor([elapsed], dtype=torch.float64, device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        elapsed = float(t.item())
    value = world * args.steps * group / ns / elapsed
    launches_per_step = (npl.launch_count(*slice_range(0), g_modp, _native.TSG_RING_MODP,
                                          NUM_PRIMES)
                         + npl.launch_count(*slice_range(0), g_or, _native.TSG_RING_OR_AND))

    # Roofline of the dominant launch: one more pass over the next slice group with a CUDA
    # event after every launch (tsg_plan_run_timed); the tree step with the largest device
    # time in either ring is the dominant launch, and its algorithmic bytes (operands read
    # once, result written once, x the slices of the group) / its event time is `achieved`.
    sp = contraction.sliced_plan
    step_s = elapsed / args.steps
    peak, peak_kind = measured_peaks()
    b, e = slice_range(args.warmup + args.steps)
    timing_passes = 2
    acc_ms = {"modp": None, "or_and": None}
    for _ in range(timing_passes):
        for name, ring, pr, ws, res, g in (
                ("modp", _native.TSG_RING_MODP, primes, ws_count, res_count, g_modp),
                ("or_and", _native.TSG_RING_OR_AND, (), ws_sat, res_sat, g_or)):
            ms = npl.run_timed(ring, pr, pool_dev, b, e, g, ws, res, False, sh)
            acc_ms[name] = ms if acc_ms[name] is None else [x + y for x, y in zip(acc_ms[name], ms)]
    # algorithmic bytes per step; a fused producer moves nothing, its consumer reads the
    # producer's operands instead of the producer's result
    fused = {"modp": npl.fused_steps(_native.TSG_RING_MODP, primes, g_modp, contraction.tree),
             "or_and": npl.fused_steps(_native.TSG_RING_OR_AND, (), g_or, contraction.tree)}
    step_bytes = {"modp": sp.step_bytes_per_slice(4, NUM_PRIMES, fused["modp"]),
                  "or_and": sp.step_bytes_per_slice(1, 1, fused["or_and"])}
    nsteps = len(step_bytes["modp"])
    ring_name, dom = max(((r, s) for r in acc_ms for s in range(nsteps)),
                         key=lambda rs: acc_ms[rs[0]][rs[1]])
    dom_ms = acc_ms[ring_name][dom] / timing_passes
    dom_bytes = step_bytes[ring_name][dom] * group
    achieved = dom_bytes / (dom_ms / 1e3) / 1e9
    step_total_ms = sum(sum(v) for v in acc_ms.values()) / timing_passes
    from tensorsat_gb300 import autotune

    traffic = dominant_traffic(ring_name, dom, g_modp if ring_name == "modp" else g_or,
                               autotune.plan_key(contraction))
    step_roofline = (sum(step_bytes["modp"]) + sum(step_bytes["or_and"])) * group / step_s / 1e9

    # end to end through the public API: host leaves in, host results out, every step
    e2e_times = []
    h2d = 2 * npl.pool_bytes
    d2h = 4 * NUM_PRIMES + 1
    for k in range(args.e2e_steps + 1):
        b, e = slice_range(args.warmup + args.steps + k)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        contraction.count(diagram, ring="modp", num_primes=NUM_PRIMES, group=g_modp,
                          slice_range=(b, e), cache_leaves=False, workspace=ws_count)
        bool(contraction.contract(diagram, group=g_or, slice_range=(b, e), cache_leaves=False,
                                  workspace=ws_sat))
        torch.cuda.synchronize()
        if k > 0:  # the first call allocates workspaces in torch's caching allocator
            e2e_times.append(time.perf_counter() - t0)
    e2e_value = world * group / ns / statistics.mean(e2e_times) if e2e_times else None

    # the whole instance: exact count and SAT bit over all slices, the slices sharded
    # across the ranks (one all-reduce per ring combines the shares)
    pg = dist.group.WORLD if dist else None
    instance = None
    if not args.no_instance:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        full_count = contraction.count(diagram, ring="modp", num_primes=NUM_PRIMES,
                                       group=g_modp, process_group=pg, workspace=ws_count)
        full_sat = bool(contraction.contract(diagram, group=g_or, process_group=pg,
                                             workspace=ws_sat))
        torch.cuda.synchronize()
        full_s = time.perf_counter() - t0
        instance = {"count": int(full_count), "sat": full_sat, "seconds": round(full_s, 3),
                    "ranks": world, "form": "GpuContraction.count + contract over all "
                    f"{ns} slices, process_group={'WORLD' if pg else None}"}
    if dpll is not None and instance is not None:
        want = dpll.get(timeout=600)
        instance["dpll_count"] = want
        if full_count != want or full_sat != (want > 0):
            raise RuntimeError(f"instance count {full_count} / SAT bit {full_sat} differ from "
                               f"the DPLL count {want}")

    batched = None
    if ragged is not None:
        # the headline's workspaces are no longer needed: give their memory to the batch
        del ws_count, ws_sat
        torch.cuda.empty_cache()
        instances, trees, expected, plan_s = ragged
        lo, hi = args.n_range
        r = ragged_measure(instances, trees, expected, args.batched_steps, args.warmup,
                           args.e2e_steps, local)
        ratio = r["e2e_value"] / r["plain_value"] if r["e2e_value"] else None
        batched = {
            "metric": RAGGED_METRIC, "value": r["value"], "unit": UNIT,
            "workload": ragged_workload_text(len(instances), lo, hi),
            "form": f"captured CUDA graphs ({r['graphs']}: one per {RAGGED_CHUNK}-instance "
                    f"chunk and ring, {RAGGED_LANES} concurrent lanes, small steps of a tree "
                    "level packed across instances) replayed, inputs resident",
            "steps": args.batched_steps, "ms_per_step": statistics.mean(r["step_ms"]),
            "unpacked": {"value": r["unpacked_value"], "unit": UNIT,
                         "gpu_launches_per_pass": r["unpacked_launches"],
                         "ms_per_step": statistics.mean(r["unpacked_step_ms"]),
                         "form": "the same graphs with one launch per tree step "
                                 "(tsg_batch_run_lanes)"},
            "plain": {"value": r["plain_value"], "unit": UNIT, "instances": len(instances),
                      "form": "GpuContraction.count + contract per instance, host leaves "
                              "uploaded and results read back by every call"},
            "e2e": {"value": r["e2e_value"], "unit": UNIT, "h2d_bytes_per_step": r["h2d"],
                    "d2h_bytes_per_step": len(instances) * (4 * NUM_PRIMES + 1),
                    "passes": r["e2e_passes"],
                    "form": "BatchContraction.serve over a stream of input batches: host "
                            "leaves in, captured graphs replayed, counts and bits out, the "
                            "host packing the next batch while the GPU runs the current one"},
            "e2e_calls": {"value": r["calls_value"], "unit": UNIT, "passes": r["calls_passes"],
                          "form": "BatchContraction.load + count/contract(graph=True) per "
                                  "batch, one call after the other"},
            "e2e_uncaptured": {"value": r["uncaptured_value"], "unit": UNIT},
            "batched_over_plain_e2e": ratio, "target_ratio": 1.5,
            "meets_target": bool(ratio is not None and ratio >= 1.5),
            "parity": f"counts and SAT bits of all {len(instances)} instances equal the "
                      "oracle's DPLL counts in the plain, batched and served forms",
            "planning_s": round(plan_s, 2), "planning_cores": cores,
            "gpu_launches_per_pass": r["launches"], "clocks": r["clocks"],
            "step_ms": [round(x, 3) for x in r["step_ms"]],
        }

    learned = learned_leg(*learned_prep) if learned_prep is not None else None

    cpu = None
    if want_cpu:
        dt, _ = cpu_sample(pool, cores, cnf, contraction, 0)
        cpu = {"value": cores / ns / dt, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"{cores} slices of {ns} (one per process, exact-integer count + "
                         f"OR-AND bit per slice, numpy einsum), {dt:.1f} s"}
    if pool is not None:
        pool.close()

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000 * step_s, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u32 residues mod 3 primes + u8 OR-AND",
            "data": "synthetic (seeded CNFInstance.random, no dataset)",
            "config": dict(workload_config(args, contraction, group),
                           slice_groups={"modp": g_modp, "or_and": g_or}),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "peak_source": peak_kind,
                         "kernel": f"tree step {dom} of the {ring_name} run (the launch with the "
                                   f"largest device time, {dom_ms:.2f} ms of "
                                   f"{step_total_ms:.1f} ms per step)",
                         "algorithmic_bytes": dom_bytes,
                         "step_achieved": step_roofline},
            "cpu_baseline": cpu,
            "e2e": ({"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d,
                     "d2h_bytes_per_step": d2h} if e2e_value is not None else None),
            "gpu_launches": launches_per_step * args.steps,
            "clocks": clocks.summary(),
            "step_ms": [round(x, 3) for x in step_ms],
            "tuning": tuning,
            "instance": instance,
            "batched": batched,
            "learned": learned,
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


# --------------------------------------------------------------------------------------
# Ragged batch: many random instances of uneven sizes


RAGGED_METRIC = "exact instances/s (SAT bit + model count), ragged batch of random 3-SAT"
RAGGED_CHUNK = 512  # instances per captured graph (the whole default batch: one per ring)
RAGGED_LANES = 32  # concurrent lanes of a batch


def ragged_instances(count: int, n_lo: int, n_hi: int):
    """n uniform in [n_lo, n_hi], clause ratio uniform in [3.5, 5.0], one generator per
    instance seeded by its index."""
    import numpy as np

    from tensorsat_gb300.lib.sat import CNFInstance

    out = []
    for i in range(count):
        g = np.random.default_rng(i)
        n = int(g.integers(n_lo, n_hi + 1))
        m = round(float(g.uniform(3.5, 5.0)) * n)
        out.append(CNFInstance.random(3, n, m, rng=g))
    return out


def _plan_instance(args):
    num_vars, clauses = args
    from tensorsat_gb300.contractions.gpu import plan_tree
    from tensorsat_gb300.lib.sat import CNFInstance

    return plan_tree(CNFInstance(num_vars, clauses).clause_diagram().wiring,
                     target_bits=TARGET_BITS, trials=1)


def _dpll_instance(args):
    """Exact model count of one instance by the oracle's DPLL counter (the checker)."""
    num_vars, clauses = args
    from oracle import finrel_oracle as orc

    return orc.dpll_count(num_vars, clauses)[0]


def ragged_plan_report(args, instances, trees, plan_s: float) -> None:
    """Algorithmic bytes of every planned instance (3-prime count + OR-AND bit, both
    operands read once and the result written once per step), summarised per n."""
    from tensorsat_gb300.contractions.gpu import GpuContraction
    from tensorsat_gb300.lang.cuda_rel import CudaRel

    by_n: dict[int, list[float]] = {}
    peak = 0
    for cnf, (tree, sliced) in zip(instances, trees):
        c = GpuContraction(CudaRel, cnf.clause_diagram().wiring, tree=tree, sliced=sliced)
        p = c.sliced_plan
        total = (p.bytes_per_slice(4, NUM_PRIMES) + p.bytes_per_slice(1, 1)) * c.num_slices
        by_n.setdefault(cnf.num_vars, []).append(total)
        peak = max(peak, c.stats()["peak_bits"])
    everything = sorted(b for bs in by_n.values() for b in bs)
    lo, hi = args.n_range
    buckets = {}
    for a in range(lo, hi + 1, 10):
        bs = sorted(b for n, v in by_n.items() if a <= n < a + 10 for b in v)
        if bs:
            buckets[f"{a}-{min(a + 9, hi)}"] = {
                "instances": len(bs), "median_bytes": bs[len(bs) // 2], "max_bytes": bs[-1],
                "sum_bytes": sum(bs)}
    print(json.dumps({
        "workload": f"ragged batch of {len(instances)} random 3-SAT instances, n uniform in "
                    f"[{lo}, {hi}], clause ratio uniform in [3.5, 5.0], seeded per instance",
        "plan_only": True, "trials": 1, "target_bits": TARGET_BITS, "peak_bits_max": peak,
        "planning_s": round(plan_s, 1), "planning_cores": min(os.cpu_count() or 1, 32),
        "total_bytes": sum(everything), "median_bytes": everything[len(everything) // 2],
        "by_n": buckets}), flush=True)


def ragged_prepare(pool, count: int, n_lo: int, n_hi: int):
    """Instances, planner trees and DPLL counts of the ragged batch. Planning is host work
    (tens of milliseconds per instance) spread over the host cores in spawned workers,
    before the calling process touches CUDA."""
    instances = ragged_instances(count, n_lo, n_hi)
    jobs = [(c.num_vars, c.clauses) for c in instances]
    t0 = time.perf_counter()
    trees = pool.map(_plan_instance, jobs, chunksize=4)
    plan_s = time.perf_counter() - t0
    expected = pool.map(_dpll_instance, jobs, chunksize=4)
    return instances, trees, expected, plan_s


def ragged_measure(instances, trees, expected, steps: int, warmup: int, e2e_steps: int,
                   device_index: int) -> dict:
    """Times the ragged batch on the GPU in three forms and checks every answer against the
    DPLL counts; returns the figures (instances/s) and the run's facts."""
    import torch

    from tensorsat_gb300 import _native
    from tensorsat_gb300.contractions.batch import BatchContraction
    from tensorsat_gb300.contractions.gpu import PRIMES_31, GpuContraction
    from tensorsat_gb300.lang.cuda_rel import CudaRel

    dev = torch.device("cuda", device_index)
    diagrams = [cnf.clause_diagram() for cnf in instances]
    primes = PRIMES_31[:NUM_PRIMES]
    chunks = [BatchContraction(CudaRel, diagrams[i: i + RAGGED_CHUNK],
                               trees=trees[i: i + RAGGED_CHUNK], lanes=RAGGED_LANES)
              for i in range(0, len(diagrams), RAGGED_CHUNK)]
    # one workspace for every graph (they replay in order on one stream); slice groups
    # sized to a fixed budget, shared by the lanes
    budget = 16 << 30
    plans = []
    need = 0
    for b in chunks:
        for ring, pr in ((_native.TSG_RING_MODP, primes), (_native.TSG_RING_OR_AND, ())):
            groups = b.groups(ring, max(1, len(pr)), budget)
            plans.append((b, ring, pr, groups))
            for packed in (True, False):
                b.packed = packed
                need = max(need, b.workspace_bytes(ring, max(1, len(pr)), groups))
            b.packed = True
    ws = torch.empty(need, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)

    def timed_graphs(packed: bool):
        """Captures one graph per chunk and ring (packed or one launch per step) and
        times `steps` passes over all of them after `warmup` passes."""
        for b in chunks:
            b.packed = packed
        graphs = [b.capture(ring, pr, groups, workspace=ws) for b, ring, pr, groups in plans]
        for b in chunks:
            b.packed = True
        torch.cuda.synchronize()
        for _ in range(warmup):
            for g in graphs:
                g.replay()
        torch.cuda.synchronize()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(steps + 1)]
        with ClockSampler(device_index) as clocks:
            ev[0].record(stream)
            for k in range(steps):
                for g in graphs:
                    g.replay()
                ev[k + 1].record(stream)
            torch.cuda.synchronize()
        GpuContraction.check_device()
        step_ms = [ev[k].elapsed_time(ev[k + 1]) for k in range(steps)]
        return graphs, step_ms, clocks

    graphs_u, step_ms_u, _ = timed_graphs(False)
    results_u = [r.cpu() for g in graphs_u for r in g.results]
    launches_u = sum(g.launches for g in graphs_u)
    del graphs_u
    graphs, step_ms, clocks = timed_graphs(True)
    results_p = [r.cpu() for g in graphs for r in g.results]
    if not all(torch.equal(a, b) for a, b in zip(results_p, results_u)):
        raise RuntimeError("packed and per-step batch runs differ")
    value = len(instances) * steps / (sum(step_ms) / 1000.0)
    unpacked_value = len(instances) * steps / (sum(step_ms_u) / 1000.0)

    # plain form: one instance per call through the public API (count + SAT bit), host
    # leaves uploaded by every call, the same instances
    plain = [GpuContraction(CudaRel, d.wiring, tree=t[0], sliced=t[1])
             for d, t in zip(diagrams, trees)]
    for c, d in zip(plain[:4], diagrams[:4]):
        c.count(d, ring="modp", num_primes=NUM_PRIMES)
        bool(c.contract(d))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    plain_counts, plain_bits = [], []
    for c, d in zip(plain, diagrams):
        plain_counts.append(int(c.count(d, ring="modp", num_primes=NUM_PRIMES,
                                        cache_leaves=False)))
        plain_bits.append(bool(c.contract(d, cache_leaves=False)))
    torch.cuda.synchronize()
    plain_value = len(plain) / (time.perf_counter() - t0)
    if plain_counts != expected or plain_bits != [e > 0 for e in expected]:
        raise RuntimeError("plain-form counts or SAT bits differ from the DPLL counts")

    # end to end, batched, uncaptured: host leaves in (uploaded again), one tsg_batch_run
    # per chunk and ring, counts and bits out
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    answers = []
    for b, i in zip(chunks, range(0, len(diagrams), RAGGED_CHUNK)):
        b.load(diagrams[i: i + RAGGED_CHUNK])
        gm = b.groups(_native.TSG_RING_MODP, NUM_PRIMES, budget)
        go = b.groups(_native.TSG_RING_OR_AND, 1, budget)
        answers.append((b.count(num_primes=NUM_PRIMES, groups=gm, workspace=ws),
                        [bool(x) for x in b.contract(groups=go, workspace=ws)]))
    torch.cuda.synchronize()
    uncaptured_value = len(diagrams) / (time.perf_counter() - t0)
    got_counts = [int(x) for counts, _ in answers for x in counts]
    got_bits = [b for _, bits in answers for b in bits]
    if got_counts != expected or got_bits != [e > 0 for e in expected]:
        raise RuntimeError("batched counts or SAT bits differ from the DPLL counts")

    # end to end, serving form: every chunk captures one graph per ring on its first call
    # (set-up, like planning); each timed pass copies every instance's host leaves into the
    # captured pools (pinned staging), replays the graphs and reads counts and bits back
    serve_groups = []
    for b in chunks:
        gm = b.groups(_native.TSG_RING_MODP, NUM_PRIMES, budget)
        go = b.groups(_native.TSG_RING_OR_AND, 1, budget)
        need = max(b.workspace_bytes(_native.TSG_RING_MODP, NUM_PRIMES, gm),
                   b.workspace_bytes(_native.TSG_RING_OR_AND, 1, go))
        if need > ws.numel():
            raise RuntimeError("serving workspace exceeds the shared workspace")
        serve_groups.append((gm, go))
        b.count(num_primes=NUM_PRIMES, groups=gm, graph=True, workspace=ws)
        b.contract(groups=go, graph=True, workspace=ws)
    torch.cuda.synchronize()
    e2e_times = []
    h2d = 0
    for k in range(e2e_steps + 1):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        copied = 0
        served = []
        for b, (gm, go), i in zip(chunks, serve_groups, range(0, len(diagrams), RAGGED_CHUNK)):
            copied += b.load(diagrams[i: i + RAGGED_CHUNK])
            served.append((b.count(num_primes=NUM_PRIMES, groups=gm, graph=True),
                           [bool(x) for x in b.contract(groups=go, graph=True)]))
        torch.cuda.synchronize()
        if served != answers:
            raise RuntimeError("graph-served answers differ from the uncaptured batch run")
        if k > 0:  # the first pass warms the pinned staging buffers
            e2e_times.append(time.perf_counter() - t0)
        h2d = copied
    calls_value = len(diagrams) / statistics.mean(e2e_times) if e2e_times else None

    # end to end, pipelined serving form (BatchContraction.serve): e2e_steps input batches
    # per chunk, the host packing batch k+1 and reading back batch k-1 while the GPU
    # contracts batch k; one warm batch per chunk allocates the pinned staging buffers
    e2e_value = None
    if e2e_steps > 0:
        def serve_chunks(passes: int) -> list:
            out = []
            for ci, (b, (gm, go), i) in enumerate(zip(chunks, serve_groups,
                                                      range(0, len(diagrams), RAGGED_CHUNK))):
                for counts, boxes in b.serve([diagrams[i: i + RAGGED_CHUNK]] * passes,
                                             NUM_PRIMES, groups=gm, sat_groups=go,
                                             workspace=ws):
                    out.append((ci, ([int(x) for x in counts], [bool(x) for x in boxes])))
            return out

        serve_chunks(1)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        served = serve_chunks(e2e_steps)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        if any(ans != answers[ci] for ci, ans in served):
            raise RuntimeError("pipelined served answers differ from the uncaptured batch run")
        e2e_value = len(diagrams) * e2e_steps / dt
    return {
        "value": value, "step_ms": step_ms, "clocks": clocks.summary(),
        "launches": sum(g.launches for g in graphs), "graphs": len(graphs),
        "unpacked_value": unpacked_value, "unpacked_launches": launches_u,
        "unpacked_step_ms": step_ms_u,
        "plain_value": plain_value, "uncaptured_value": uncaptured_value,
        "e2e_value": e2e_value, "e2e_passes": e2e_steps, "h2d": h2d,
        "calls_value": calls_value, "calls_passes": len(e2e_times),
    }


def ragged_workload_text(count: int, lo: int, hi: int) -> str:
    return (f"ragged batch of {count} random 3-SAT instances, n uniform in [{lo}, {hi}], "
            f"clause ratio uniform in [3.5, 5.0], seeded per instance")


def run_ragged(args) -> None:
    lo, hi = args.n_range
    # The planner calls the native library's host code: load (and if needed build) it here
    # once, not in every worker.
    from tensorsat_gb300 import _native

    _native.lib()
    if args.plan_only:
        instances = ragged_instances(args.instances, lo, hi)
        jobs = [(c.num_vars, c.clauses) for c in instances]
        t_plan = time.perf_counter()
        with cpu_pool(max(1, min(os.cpu_count() or 1, 32))) as pool:
            trees = pool.map(_plan_instance, jobs, chunksize=4)
        ragged_plan_report(args, instances, trees, time.perf_counter() - t_plan)
        return
    with cpu_pool(max(1, min(os.cpu_count() or 1, 32))) as pool:
        instances, trees, expected, _ = ragged_prepare(pool, args.instances, lo, hi)

    import torch

    torch.cuda.set_device(0)
    r = ragged_measure(instances, trees, expected, args.steps, args.warmup, args.e2e_steps, 0)
    line = {
        "metric": RAGGED_METRIC, "value": r["value"], "unit": UNIT, "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": statistics.mean(r["step_ms"]), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32 residues mod 3 primes + u8 OR-AND",
        "data": "synthetic (seeded CNFInstance.random per instance, no dataset)",
        "config": {"workload": ragged_workload_text(len(instances), lo, hi),
                   "instances": len(instances), "n_range": [lo, hi],
                   "graphs": r["graphs"], "instances_per_graph": RAGGED_CHUNK,
                   "l2": "not flushed: small instances are L2-resident by design"},
        "parity": f"counts and SAT bits of all {len(instances)} instances equal the "
                  "oracle's DPLL counts (plain, batched and served forms)",
        "plain": {"value": r["plain_value"], "unit": UNIT, "sample": len(instances),
                  "form": "GpuContraction.count + contract per instance"},
        "e2e": ({"value": r["e2e_value"], "unit": UNIT, "h2d_bytes_per_step": r["h2d"],
                 "d2h_bytes_per_step": len(instances) * (4 * NUM_PRIMES + 1),
                 "form": "BatchContraction.serve over a stream of input batches per chunk: "
                         "host leaves in, captured graphs replayed, counts and bits out, "
                         "the host packing the next batch while the GPU runs the current one",
                 "passes": r["e2e_passes"]} if r["e2e_value"] is not None else None),
        "e2e_calls": {"value": r["calls_value"], "unit": UNIT,
                      "form": "BatchContraction.load + count/contract(graph=True) per chunk"},
        "e2e_uncaptured": {"value": r["uncaptured_value"], "unit": UNIT,
                           "form": "BatchContraction.count + contract per chunk, no graph"},
        "gpu_launches": r["launches"] * args.steps,
        "unpacked": {"value": r["unpacked_value"], "unit": UNIT,
                     "gpu_launches_per_pass": r["unpacked_launches"],
                     "form": "the same graphs with one launch per tree step"},
        "clocks": r["clocks"],
        "step_ms": [round(x, 3) for x in r["step_ms"]],
    }
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------------------------------
# Learned cost model: trained on the solver's own measurements, evaluated on n=60


def _candidates_job(args):
    num_vars, clauses, count = args[:3]
    settings = args[3] if len(args) > 3 else None
    from tensorsat_gb300 import costmodel
    from tensorsat_gb300.lib.sat import CNFInstance

    return costmodel.candidate_trees(CNFInstance(num_vars, clauses).clause_diagram().wiring,
                                     count, settings=settings)


def candidates_parallel(pool, instances, count: int, parts: int = 8):
    """The planner candidates of every instance, each instance's settings split over
    ``parts`` workers (the planner's usual choice stays first)."""
    from tensorsat_gb300 import costmodel

    return costmodel.cnf_candidates(pool, instances, count, parts)


COSTMODEL_FILE = ROOT / "plans" / "costmodel_n60.npz"


def costmodel_heldout(count: int):
    """Held-out n=60, m=256 instances of the cost model's evaluation (seeds 10000 on)."""
    from tensorsat_gb300.lib.sat import CNFInstance

    return [CNFInstance.random(3, N_VARS, N_CLAUSES, rng=10_000 + j) for j in range(count)]


def costmodel_measure(instances, cands, group: int):
    """Every candidate tree of every instance: (contraction, tree graph, measured device
    ms per slice) per candidate, per instance."""
    from tensorsat_gb300 import costmodel
    from tensorsat_gb300.contractions.gpu import PRIMES_31, GpuContraction
    from tensorsat_gb300.lang.cuda_rel import CudaRel

    primes = PRIMES_31[:NUM_PRIMES]
    rows = []
    for inst, cs in zip(instances, cands):
        d = inst.clause_diagram()
        per = []
        for tree, sl in cs:
            c = GpuContraction(CudaRel, d.wiring, tree=tree, sliced=sl)
            ms = costmodel.measure(c, d, primes, group, passes=1)
            per.append((c, costmodel.tree_graph(c, min(group, c.num_slices), primes), ms))
        rows.append(per)
    return rows


def costmodel_evaluate(model, held, rows, dpll, exact_checks: int) -> dict:
    """Prediction error on the held-out trees, and per instance the measured device time
    of the tree the model picks against the planner's pick (candidate 0) and the best."""
    import numpy as np

    from tensorsat_gb300 import costmodel

    hg = [gph for per in rows for _, gph, _ in per]
    hy = np.asarray([math.log(ms) for per in rows for _, _, ms in per])
    pred = np.concatenate([model.predict(costmodel.make_batch(hg[i: i + 64], model.device))
                           for i in range(0, len(hg), 64)])
    err = np.abs(pred - hy)
    picks, chosen = [], []
    k = 0
    for per in rows:
        cost_pred = [math.exp(pred[k + j]) * per[j][0].num_slices for j in range(len(per))]
        cost_meas = [per[j][2] * per[j][0].num_slices for j in range(len(per))]
        k += len(per)
        j = int(np.argmin(cost_pred))
        chosen.append(per[j][0])
        picks.append((cost_meas[j], cost_meas[0], min(cost_meas)))
    exact = [int(c.count(inst.clause_diagram(), ring="modp", num_primes=NUM_PRIMES)) == want
             for inst, c, want in list(zip(held, chosen, dpll))[:exact_checks]]
    return {
        "mean_abs_log_error": float(err.mean()), "median_abs_log_error": float(np.median(err)),
        "within_20pct": float(np.mean(err < math.log(1.2))),
        "heldout_instances": len(held), "heldout_trees": len(hg),
        "model_pick_over_best": float(np.mean([m / b for m, _, b in picks])),
        "planner_pick_over_best": float(np.mean([p / b for _, p, b in picks])),
        "learned_over_plain": float(np.mean([p / m for m, p, _ in picks])),
        "learned_over_plain_total": float(sum(p for _, p, _ in picks) / sum(m for m, _, _ in picks)),
        "picked_trees_exact": exact,
    }


def learned_leg(held, cands, dpll_held, group: int = 16) -> dict:
    """The learned path on held-out n=60 instances: the committed cost model ranks each
    instance's planner candidates by predicted device time (per-slice prediction x slices)
    and picks the cheapest; the planner's own tree (candidate 0) is the plain path and the
    fallback whenever the model ranks it first. Both picks are measured on the device and
    the picked tree's full count is checked against DPLL on two instances."""
    import numpy as np

    from tensorsat_gb300 import costmodel
    from tensorsat_gb300.contractions.gpu import PRIMES_31, GpuContraction
    from tensorsat_gb300.lang.cuda_rel import CudaRel

    primes = PRIMES_31[:NUM_PRIMES]
    model = costmodel.CostModel(seed=0)
    model.load_state(dict(np.load(COSTMODEL_FILE)))
    rows, err, exact = [], [], []
    t0 = time.perf_counter()
    for i, (inst, cs) in enumerate(zip(held, cands)):
        d = inst.clause_diagram()
        cons = [GpuContraction(CudaRel, d.wiring, tree=t, sliced=sl) for t, sl in cs]
        graphs = [costmodel.tree_graph(c, min(group, c.num_slices), primes) for c in cons]
        pred = model.predict(costmodel.make_batch(graphs, model.device))
        cost_pred = [math.exp(p) * c.num_slices for p, c in zip(pred, cons)]
        j = int(np.argmin(cost_pred))
        ms = {k: costmodel.measure(cons[k], d, primes, group, passes=1) for k in {0, j}}
        err += [abs(pred[k] - math.log(v)) for k, v in ms.items()]
        plain, learned = ms[0] * cons[0].num_slices, ms[j] * cons[j].num_slices
        rows.append((plain, learned, j, cons[j], d))
    # the picked trees of the two instances with the shortest learned runs count exactly
    for i in sorted(range(len(rows)), key=lambda i: rows[i][1])[:2]:
        _, _, _, c, d = rows[i]
        got = c.count(d, ring="modp", num_primes=NUM_PRIMES)
        exact.append({"instance": 10_000 + i, "count": int(got), "dpll": int(dpll_held[i]),
                      "equal": int(got) == int(dpll_held[i])})
    rows = [r[:3] for r in rows]
    return {
        "metric": "device ms per instance, learned tree vs planner tree (3-SAT n=60 m=256)",
        "instances": len(held), "candidates_per_instance": [len(cs) for cs in cands],
        "learned_over_plain": float(np.mean([p / q for p, q, _ in rows])),
        "learned_over_plain_total": float(sum(p for p, _, _ in rows) / sum(q for _, q, _ in rows)),
        "picked_planner_tree": sum(1 for *_, j in rows if j == 0),
        "plain_ms_per_instance": [round(p, 1) for p, _, _ in rows],
        "learned_ms_per_instance": [round(q, 1) for _, q, _ in rows],
        "abs_log_error_measured_picks": float(np.mean(err)),
        "picked_trees_exact": exact, "target_ratio": 1.5,
        "meets_target": bool(sum(p for p, _, _ in rows) >= 1.5 * sum(q for _, q, _ in rows)),
        "seconds": round(time.perf_counter() - t0, 1),
        "form": "committed cost model (plans/costmodel_n60.npz) ranks the planner's candidate "
                "trees per held-out instance (seeds 10000 on); device time per instance = "
                f"measured ms per slice (tsg_plan_run_timed, {group} slices, 3-prime count + "
                "OR-AND) x slices",
    }


def run_costmodel_eval(args) -> None:
    """Evaluates the committed cost model (no training) on --cm-heldout held-out n=60,
    m=256 instances (seeds 10000 on), 4 planner candidates each, every candidate measured
    on the device: prediction error, and the measured device time of the model's pick
    against the planner's pick and the best candidate."""
    import numpy as np

    from tensorsat_gb300 import _native

    _native.lib()
    held = costmodel_heldout(args.cm_heldout)
    cores = os.cpu_count() or 1
    t0 = time.perf_counter()
    with cpu_pool(cores) as pool:
        cand_held = pool.map(_candidates_job, [(c.num_vars, c.clauses, 4) for c in held],
                             chunksize=4)
        dpll_held = pool.map(_dpll_instance, [(c.num_vars, c.clauses) for c in held[:4]])
    plan_s = time.perf_counter() - t0

    import torch

    from tensorsat_gb300 import costmodel

    torch.cuda.set_device(0)
    group = 16
    model = costmodel.CostModel(seed=0)
    model.load_state(dict(np.load(COSTMODEL_FILE)))
    t0 = time.perf_counter()
    rows = costmodel_measure(held, cand_held, group)
    measure_s = time.perf_counter() - t0
    ev = costmodel_evaluate(model, held, rows, dpll_held, 4)
    line = {
        "metric": "committed cost model on held-out 3-SAT n=60 m=256 instances: "
                  "|log predicted - log measured| device time per slice",
        "value": ev["mean_abs_log_error"], "unit": "mean abs log error",
        "higher_is_better": False, **ev,
        "seconds": {"planning": round(plan_s, 1), "measuring": round(measure_s, 1)},
        "config": {"weights": "plans/costmodel_n60.npz", "candidates_per_instance": 4,
                   "measure": f"tsg_plan_run_timed, {group} slices, 3-prime count + OR-AND"},
    }
    print(json.dumps(line), flush=True)


def run_costmodel(args) -> None:
    """Trains the cost model on measured candidate trees of random 3-SAT instances (n
    uniform in [24, 56]) and evaluates it on held-out n=60, m=256 instances: prediction
    error of the device time per slice, and the measured time of the tree it picks per
    instance against the planner's pick and the best candidate."""
    import numpy as np

    from tensorsat_gb300 import _native

    _native.lib()
    from tensorsat_gb300.lib.sat import CNFInstance

    g = np.random.default_rng(1)
    train = []
    for i in range(args.cm_train):
        n = int(g.integers(24, 57))
        m = round(float(g.uniform(3.8, 4.6)) * n)
        train.append(CNFInstance.random(3, n, m, rng=1000 + i))
    held = costmodel_heldout(args.cm_heldout)
    cores = os.cpu_count() or 1
    t0 = time.perf_counter()
    with cpu_pool(cores) as pool:
        cand_train = pool.map(_candidates_job, [(c.num_vars, c.clauses, 5) for c in train])
        cand_held = pool.map(_candidates_job, [(c.num_vars, c.clauses, 4) for c in held])
        dpll_held = pool.map(_dpll_instance, [(c.num_vars, c.clauses) for c in held[:4]])
    plan_s = time.perf_counter() - t0

    import torch

    from tensorsat_gb300 import costmodel

    torch.cuda.set_device(0)
    group = 16
    t0 = time.perf_counter()
    rows_train = costmodel_measure(train, cand_train, group)
    rows_held = costmodel_measure(held, cand_held, group)
    measure_s = time.perf_counter() - t0
    graphs = [gph for per in rows_train for _, gph, _ in per]
    y = [math.log(ms) for per in rows_train for _, _, ms in per]
    model = costmodel.CostModel(seed=0)
    t0 = time.perf_counter()
    hist = model.fit(graphs, y, epochs=args.cm_epochs, batch_trees=64, lr=2e-3)
    train_s = time.perf_counter() - t0
    ev = costmodel_evaluate(model, held, rows_held, dpll_held, 4)
    if args.cm_out:
        np.savez(args.cm_out, **model.state())
    line = {
        "metric": "learned cost model: |log predicted - log measured| device time per slice, "
                  "held-out 3-SAT n=60 m=256 trees",
        "value": ev["mean_abs_log_error"], "unit": "mean abs log error",
        "higher_is_better": False, **ev, "train_trees": len(graphs),
        "loss_first_last": [hist[0], hist[-1]],
        "seconds": {"planning": round(plan_s, 1), "measuring": round(measure_s, 1),
                    "training": round(train_s, 1)},
        "config": {"hidden": costmodel.HIDDEN, "layers": costmodel.LAYERS, "epochs": args.cm_epochs,
                   "dtype": "bf16 weights/activations, fp32 accumulation (tcgen05 kind::f16)",
                   "measure": f"tsg_plan_run_timed, {group} slices, 3-prime count + OR-AND"},
    }
    print(json.dumps(line), flush=True)


def run_costmodel_gemm(args) -> None:
    """Times the cost model's tensor-core layer GEMM (node rows x 128 weights, K = 128,
    bias + ReLU, BF16 out) at 2^19 node rows (operands and result larger than L2), and
    the same product through cuBLAS (torch.nn.functional.linear) for comparison."""
    import torch

    from tensorsat_gb300 import _device, _native

    lib = _native.lib()
    torch.cuda.set_device(0)
    m, n, k = 1 << 19, 128, 128
    g = torch.Generator(device="cuda").manual_seed(0)
    a = torch.randn(m, k, device="cuda", generator=g).to(torch.bfloat16)
    w = torch.randn(n, k, device="cuda", generator=g).to(torch.bfloat16)
    bias = torch.randn(n, device="cuda", generator=g)
    out = torch.empty(m, n, device="cuda", dtype=torch.bfloat16)
    stream = _device.stream_handle()

    def ours():
        _native.check(lib.tsg_cm_gemm_bf16(m, n, k, a.data_ptr(), w.data_ptr(), bias.data_ptr(),
                                           1, out.data_ptr(), n, 0, stream))

    bias16 = bias.to(torch.bfloat16)

    def cublas():
        torch.relu(torch.nn.functional.linear(a, w, bias16))

    def timed(fn, steps):
        for _ in range(max(3, args.warmup)):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(steps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps

    steps = max(args.steps, 20)
    want = torch.relu(a.float() @ w.float().T + bias)
    forms = {}
    for mode, name in ((1, "staged"), (0, "tma")):
        _native.check(lib.tsg_cm_set_gemm_mode(mode))
        out.zero_()
        t = timed(ours, steps)
        _native.check(lib.tsg_cm_take_error(stream))
        forms[name] = {"ms_per_launch": t,
                       "max_rel_error_vs_fp32": float((out.float() - want).abs().max()
                                                      / want.abs().max())}
    _native.check(lib.tsg_cm_set_gemm_mode(0))
    ms = forms["tma"]["ms_per_launch"]
    err = forms["tma"]["max_rel_error_vs_fp32"]
    ms_cublas = timed(cublas, steps)
    flops = 2.0 * m * n * k
    nbytes = 2.0 * (m * k + n * k + m * n) + 4 * n
    peak, kind = measured_peaks()
    line = {
        "metric": "cost-model layer GEMM (TMA tensor loads, tcgen05.mma kind::f16, TMEM "
                  "accumulator, bias+ReLU epilogue), node rows x 128 x 128",
        "value": nbytes / ms / 1e6, "unit": "GB/s", "higher_is_better": True,
        "ms_per_launch": ms, "steps": steps, "warmup": max(3, args.warmup),
        "tflops": flops / ms / 1e9, "cublas_ms_per_launch": ms_cublas,
        "forms": forms,
        "over_cublas": ms_cublas / ms, "max_rel_error_vs_fp32": err,
        "roofline": {"bound": "hbm", "achieved": nbytes / ms / 1e6, "peak": peak,
                     "unit": "GB/s", "frac": nbytes / ms / 1e6 / peak, "peak_source": kind,
                     "algorithmic_bytes": nbytes},
        "config": {"workload": f"{m} x {n} x {k} BF16, FP32 accumulation, BF16 out",
                   "l2": "operands and result larger than L2"},
    }
    print(json.dumps(line), flush=True)


def main() -> None:
    args = parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "ragged":
        run_ragged(args)
    elif args.workload == "costmodel":
        run_costmodel(args)
    elif args.workload == "costmodel-eval":
        run_costmodel_eval(args)
    elif args.workload == "costmodel-gemm":
        run_costmodel_gemm(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
