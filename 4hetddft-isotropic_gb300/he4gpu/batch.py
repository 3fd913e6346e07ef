"""Many uneven collision runs advancing together.

32 seeded collision runs (he4gpu.initial.batch_cases: N log-uniform in
[300, 3000], grids of 96^3, 128^3 or 160^3, Xe at 100-600 m/s, impact
parameter in [0, R]) are advanced together in the mixed-precision form: one
stream per run, every predictor-corrector step replayed from a CUDA graph,
all runs' launches interleaved step by step (he4g_step_many), so that small
grids fill the device together; and as one CUDA graph per batch step over all
runs (he4g_batch_step). The same runs stepped one after another in
plain FP64 are the baseline. Reports aggregate grid-point updates/s of both,
and checks that one run's result in the batch equals its result alone.

  python -m he4gpu.batch --runs 32 --steps 20
"""
import argparse
import json
import sys
import time

import numpy as np

from . import batch_cases, state_for, step_many
from . import serve as _serve
from .serve import make_run

MIXED = 1
FP64 = 0


def batched(cases, steps, warm=5):
    """The runs advanced together twice over: per-stream (he4g_step_many: one
    graph launch per run and step) and as one graph per batch step
    (he4g_batch_step). The graphs of both paths are captured in untimed
    steps first (each run's slot arrangements recur every 10 steps)."""
    from . import Batch
    runs = []
    for meta in cases:
        run, cfg = make_run(meta, MIXED, graphs=True)
        psi, r, v = state_for(meta)
        run.set_state(psi, r, v)
        runs.append((run, cfg.nx * cfg.ny * cfg.nz))
    handles = [r for r, _ in runs]
    step_many(handles, max(warm, 3 + 10))
    t0 = time.perf_counter()
    step_many(handles, steps)
    dt_streams = time.perf_counter() - t0
    batch = Batch(handles)
    batch.step(10)
    t0 = time.perf_counter()
    batch.step(steps)
    dt_graph = time.perf_counter() - t0
    ngraphs = batch.graphs
    batch.close()
    points = sum(p for _, p in runs)
    first = runs[0][0]
    res0 = (first.psi, first.impurity()[0], first.steps_taken)
    for r, _ in runs:
        r.close()
    return {"runs": len(cases), "steps": steps,
            "per_stream": {"wall_s": dt_streams, "grid_point_updates_per_s": points * steps / dt_streams},
            "one_graph_per_batch_step": {"wall_s": dt_graph, "grid_point_updates_per_s": points * steps / dt_graph,
                                         "graphs_captured": ngraphs},
            "grid_point_updates_per_s": points * max(steps / dt_streams, steps / dt_graph),
            "steps_per_s_per_run": max(steps / dt_streams, steps / dt_graph)}, res0


def sequential_fp64(cases, steps, warm=4):
    total_s = 0.0
    updates = 0
    for meta in cases:
        run, cfg = make_run(meta, FP64, graphs=False)
        psi, r, v = state_for(meta)
        run.set_state(psi, r, v)
        run.step(warm)
        ms = run.step_timed(steps)
        total_s += ms / 1e3
        updates += cfg.nx * cfg.ny * cfg.nz * steps
        run.close()
    return {"runs": len(cases), "steps": steps, "device_s": total_s, "grid_point_updates_per_s": updates / total_s}


def alone(meta, steps_total):
    run, _ = make_run(meta, MIXED, graphs=False)
    psi, r, v = state_for(meta)
    run.set_state(psi, r, v)
    run.step(steps_total)
    out = (run.psi, run.impurity()[0])
    run.close()
    return out


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--runs", type=int, default=32)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--fused-planes", action="store_true", help="keep the fused y/x plane kernels")
    args = ap.parse_args(argv)
    _serve.KEEP_FUSED_PLANES = args.fused_planes
    cases = batch_cases(args.runs, seed=args.seed)
    b, res0 = batched(cases, args.steps)
    s = sequential_fp64(cases, args.steps)
    a = alone(cases[0], res0[2])
    same = bool(np.array_equal(a[0], res0[0]) and np.array_equal(a[1], res0[1]))
    grids = {}
    for m in cases:
        grids[m["nx"]] = grids.get(m["nx"], 0) + 1
    out = {"batched_mixed": b, "sequential_fp64": s,
           "ratio": b["grid_point_updates_per_s"] / s["grid_point_updates_per_s"],
           "alone_equals_batched": same, "grids": grids, "seed": args.seed, "fused_planes": args.fused_planes}
    print(json.dumps(out), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
