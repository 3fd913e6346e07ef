"""Continuous-batching request loop for collision jobs.

Jobs arrive as a seeded Poisson stream. The loop admits an arrived job when
its device footprint (he4g_footprint) fits the HBM budget and a slot is free.
An admitted job's psi and history stay resident until it completes. All
resident jobs advance together, a chunk of steps at a time (he4g_step_many:
one stream per job, predictor-corrector steps replayed from CUDA graphs), so
that jobs that arrive while others run share the device. A finished job is
evicted, which frees its memory for the next arrival.

The report gives jobs/h, p50/p99 per-step latency (a resident job's share of
a chunk: chunk wall time / steps in the chunk) and p50/p99 time to completion
(arrival to last step). The same stream is then served one job at a time in
plain FP64 on the same GPU, for real: a FIFO single server that waits for
each arrival and runs the job to completion. Every job's final total energy
and norm in the mixed form are compared with its FP64 twin's (|dE/E| < 1e-6
and norm drift < 1e-8 is the bar). `--baseline modelled` replaces the FP64
run by a FIFO model over per-grid FP64 step times measured here.

  python -m he4gpu.serve --jobs 200 --step-scale 0.1
"""
import argparse
import json
import sys
import time

import numpy as np

from . import He4gError, Run, config_for_case, default_config, footprint, serve_stream, state_for, step_many

MIXED = 1
FP64 = 0


# FFT tile shapes tuned once per (grid, precision, sharing) and reused by later runs
_TILES = {}

# tiles[4] bit of the fused y/x plane kernels (thread-block clusters)
FUSED_PLANES = 16
# whether runs that share the GPU keep them (--fused-planes)
KEEP_FUSED_PLANES = False


def make_run(meta, precision, graphs=True, tune=True, shared=True, fused_planes=None):
    """A run for `meta`, with FFT tiles tuned once per grid. shared: the run
    will advance together with others (batch, serving); the autotuner times
    each pass alone, where the fused plane kernels can win, but with many
    runs on the GPU their cluster-wide barriers and large blocks cost more
    than the bytes they save, so shared runs leave them out unless
    fused_planes (default: KEEP_FUSED_PLANES) is set."""
    if fused_planes is None:
        fused_planes = KEEP_FUSED_PLANES
    kw, tk = config_for_case(meta)
    cfg = default_config(meta["nx"], meta["ny"], meta["nz"], meta["xmax"], meta["ymax"], meta["zmax"],
                         precision=precision, **kw)
    # k-space tables built on the device: admission skips the host loop over
    # the half grid (0.4 s at 256^3 on one core)
    run = Run(cfg, selec=tk["selec"], r_cutoff=tk["r_cutoff"], umax=tk["umax"], device_tables=True)
    if tune:
        drop = shared and not fused_planes
        key = (cfg.nx, cfg.ny, cfg.nz, precision, drop)
        if key not in _TILES:
            t = tuple(run.autotune())
            _TILES[key] = t[:4] + (t[4] & ~FUSED_PLANES,) if drop else t
        run.tiles = _TILES[key]
    if graphs:
        run.enable_graphs(True)
    return run, cfg


def job_config(meta, precision):
    kw, _ = config_for_case(meta)
    return default_config(meta["nx"], meta["ny"], meta["nz"], meta["xmax"], meta["ymax"], meta["zmax"],
                          precision=precision, **kw)


def pct(xs, q):
    return float(np.percentile(np.asarray(xs, dtype=float), q)) if xs else None


def final_state(run, meta):
    """The job's last total energy, the sum of its components' magnitudes
    (the energy scale: etot is a difference of large terms and can be small)
    and its norm (energy.f90, sum(den)*dxyz)."""
    e = run.energy()
    scale = sum(abs(e[k]) for k in ("ekin4", "elj4", "ecor4", "ealphas", "esolid", "eext", "ekinx", "eHeX"))
    return {"etot": e["etot"], "escale": scale, "norm": run.observables(meta["n4"])["npart"]}


def serve(stream, hbm_budget, max_active=64, chunk=16, precision=MIXED, keep_results=(0,), state_fn=state_for):
    """Runs the request loop over `stream` [(arrival_s, meta)] in wall-clock
    time; returns (report, results of the jobs listed in keep_results). The
    report's "finals" holds every job's final energy and norm. state_fn(meta)
    gives a job's (psi, rimp, vimp). A job whose density check or impurity
    table check fails inside a chunk (he4g_step_many stops that run only) is
    evicted and listed in the report's "failed" with its error; the other
    jobs continue."""
    pending = list(enumerate(stream))
    finals = {}
    failed = []
    max_resident = 0
    active = []  # dicts: id, run, left, arrival, admitted, bytes, points
    step_lat = []
    done = []
    kept = {}
    used = 0
    t0 = time.perf_counter()
    grid_updates = 0
    while pending or active:
        now = time.perf_counter() - t0
        # admit arrived jobs in arrival order while memory and slots allow
        while pending and pending[0][1][0] <= now and len(active) < max_active:
            jid, (arr, meta) = pending[0]
            need = footprint(job_config(meta, precision))
            if used + need > hbm_budget and active:
                break
            pending.pop(0)
            run, cfg = make_run(meta, precision)
            psi, r, v = state_fn(meta)
            try:
                run.set_state(psi, r, v)
            except He4gError as err:  # the first evaluation already fails
                run.close()
                failed.append({"id": jid, "code": err.code, "error": str(err)})
                continue
            used += need
            active.append({"id": jid, "run": run, "left": meta["steps"], "arrival": arr,
                           "admitted": time.perf_counter() - t0, "bytes": need,
                           "points": cfg.nx * cfg.ny * cfg.nz, "meta": meta})
            max_resident = max(max_resident, len(active))
        if not active:
            # idle until the next arrival
            wait = pending[0][1][0] - (time.perf_counter() - t0)
            if wait > 0:
                time.sleep(min(wait, 0.05))
            continue
        k = min(chunk, min(a["left"] for a in active))
        ts = time.perf_counter()
        try:
            step_many([a["run"] for a in active], k)
        except He4gError:
            # evict the runs whose checks failed; the others took their k steps
            bad = []
            for a in active:
                code, msg = a["run"].health()
                if code:
                    bad.append(a)
                    failed.append({"id": a["id"], "code": code, "error": msg})
            if not bad:
                raise
            for a in bad:
                a["run"].close()
                used -= a["bytes"]
            active = [a for a in active if a not in bad]
        dt = time.perf_counter() - ts
        for a in active:
            a["left"] -= k
            step_lat.extend([dt / k] * k)
            grid_updates += a["points"] * k
        finished = [a for a in active if a["left"] == 0]
        active = [a for a in active if a["left"] > 0]
        tnow = time.perf_counter() - t0
        for a in finished:
            finals[a["id"]] = final_state(a["run"], a["meta"])
            if a["id"] in keep_results:
                rr, vv, _ = a["run"].impurity()
                kept[a["id"]] = {"psi": a["run"].psi, "rimp": rr, "vimp": vv, "etot": a["run"].energy()["etot"]}
            a["run"].close()
            used -= a["bytes"]
            done.append({"id": a["id"], "arrival": a["arrival"], "finish": tnow, "ttc": tnow - a["arrival"],
                         "queue": a["admitted"] - a["arrival"], "steps": a["meta"]["steps"],
                         "grid": a["meta"]["nx"]})
    makespan = time.perf_counter() - t0
    ttc = [d["ttc"] for d in done]
    rep = {
        "jobs": len(done),
        "makespan_s": makespan,
        "jobs_per_h": len(done) / makespan * 3600.0,
        "step_latency_ms_p50": 1e3 * pct(step_lat, 50),
        "step_latency_ms_p99": 1e3 * pct(step_lat, 99),
        "ttc_s_p50": pct(ttc, 50),
        "ttc_s_p99": pct(ttc, 99),
        "grid_point_updates_per_s": grid_updates / makespan,
        "precision": "mixed" if precision == MIXED else "fp64",
        "max_resident": max_resident,
        "finals": finals,
        "failed": failed,
    }
    return rep, kept


def fp64_step_seconds(grids, steps=6):
    """Measured FP64 step time per grid size (one run alone, direct launches)."""
    out = {}
    from .initial import make_meta
    for g in grids:
        meta = make_meta(g, 0.42, min(5000.0, ((g * 0.42 / 2 - 8) / 2.22) ** 3 * 0.6), "Xe", 0.3, 3.0)
        run, _ = make_run(meta, FP64, graphs=False)
        psi, r, v = state_for(meta)
        run.set_state(psi, r, v)
        run.step(4)
        ms = run.step_timed(steps)
        out[g] = ms / 1e3 / steps
        run.close()
    return out


def one_at_a_time_measured(stream, precision=FP64):
    """The same arrivals served for real by a FIFO single server in plain
    FP64: each job waits for its arrival and for the job before it, then runs
    all its steps alone on the GPU (graph replay, tuned tiles). Returns the
    report with every job's final energy and norm."""
    t0 = time.perf_counter()
    ttc, steps_lat, finals = [], [], {}
    for jid, (arr, meta) in enumerate(stream):
        wait = arr - (time.perf_counter() - t0)
        if wait > 0:
            time.sleep(wait)
        run, _ = make_run(meta, precision, shared=False)
        psi, r, v = state_for(meta)
        run.set_state(psi, r, v)
        ts = time.perf_counter()
        run.step(meta["steps"])
        steps_lat.append((time.perf_counter() - ts) / meta["steps"])
        finals[jid] = final_state(run, meta)
        run.close()
        ttc.append(time.perf_counter() - t0 - arr)
    makespan = time.perf_counter() - t0
    return {"jobs": len(stream), "makespan_s": makespan, "jobs_per_h": len(stream) / makespan * 3600.0,
            "step_latency_ms_p50": 1e3 * pct(steps_lat, 50), "step_latency_ms_p99": 1e3 * pct(steps_lat, 99),
            "ttc_s_p50": pct(ttc, 50), "ttc_s_p99": pct(ttc, 99), "precision": "fp64", "measured": True,
            "finals": finals}


def pretune(stream, precision, shared=True):
    """Tunes the FFT tiles of every grid of the stream before a timed run,
    so that neither server pays the tuner inside its timeline."""
    for g in sorted({(m["nx"], m["ny"], m["nz"]) for _, m in stream}):
        meta = next(m for _, m in stream if (m["nx"], m["ny"], m["nz"]) == g)
        run, _ = make_run(meta, precision, graphs=False, shared=shared)
        run.close()


def compare_finals(mixed, fp64):
    """Per job: |E_mixed - E_fp64| / |E_fp64|, the same difference over the
    job's energy scale (sum of the components' magnitudes), and
    |N_mixed - N_fp64| / N_fp64."""
    jobs = [j for j in fp64 if j in mixed]
    de = {j: abs(mixed[j]["etot"] - fp64[j]["etot"]) / abs(fp64[j]["etot"]) for j in jobs}
    ds = {j: abs(mixed[j]["etot"] - fp64[j]["etot"]) / fp64[j]["escale"] for j in jobs}
    dn = {j: abs(mixed[j]["norm"] - fp64[j]["norm"]) / abs(fp64[j]["norm"]) for j in jobs}
    return {"jobs_compared": len(de), "dE_rel_max": max(de.values()) if de else None,
            "dE_rel_p50": pct(list(de.values()), 50), "dE_over_scale_max": max(ds.values()) if ds else None,
            "norm_rel_max": max(dn.values()) if dn else None,
            "jobs_within_dE_1e-6": sum(1 for v in de.values() if v < 1e-6),
            "jobs_within_norm_1e-8": sum(1 for v in dn.values() if v < 1e-8)}


def one_at_a_time(stream, step_s):
    """FIFO single server in plain FP64 over the same arrivals, modelled from
    per-grid step times."""
    t = 0.0
    ttc = []
    for arr, meta in stream:
        start = max(t, arr)
        t = start + meta["steps"] * step_s[meta["nx"]]
        ttc.append(t - arr)
    return {"jobs": len(stream), "makespan_s": t, "jobs_per_h": len(stream) / t * 3600.0,
            "step_latency_ms_by_grid": {str(g): 1e3 * s for g, s in step_s.items()},
            "ttc_s_p50": pct(ttc, 50), "ttc_s_p99": pct(ttc, 99), "precision": "fp64"}


def alone_vs_mix(stream, kept, precision=MIXED):
    """Re-runs the kept jobs alone and compares their final state bit for bit."""
    out = {}
    for jid, res in kept.items():
        meta = stream[jid][1]
        run, _ = make_run(meta, precision)
        psi, r, v = state_for(meta)
        run.set_state(psi, r, v)
        run.step(meta["steps"])
        same = bool(np.array_equal(run.psi, res["psi"]) and np.array_equal(run.impurity()[0], res["rimp"]))
        out[str(jid)] = {"identical": same, "etot_alone": run.energy()["etot"], "etot_mix": res["etot"]}
        run.close()
    return out


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--jobs", type=int, default=200)
    ap.add_argument("--rate", type=float, default=4.0, help="arrivals per second")
    ap.add_argument("--step-scale", type=float, default=1.0, help="scales each job's 500-5000 steps")
    ap.add_argument("--chunk", type=int, default=16)
    ap.add_argument("--max-active", type=int, default=64)
    ap.add_argument("--hbm-gb", type=float, default=0.0, help="budget; 0 = 90%% of the free memory")
    ap.add_argument("--seed", type=int, default=7)
    ap.add_argument("--fused-planes", action="store_true", help="keep the fused y/x plane kernels")
    ap.add_argument("--baseline", default="measured", choices=["measured", "modelled"],
                    help="the one-at-a-time FP64 server: run for real, or modelled from per-grid step times")
    args = ap.parse_args(argv)
    global KEEP_FUSED_PLANES
    KEEP_FUSED_PLANES = args.fused_planes
    stream = serve_stream(args.jobs, seed=args.seed, rate_per_s=args.rate, step_scale=args.step_scale)
    if args.hbm_gb > 0:
        budget = int(args.hbm_gb * 1e9)
    else:
        import torch
        free, _ = torch.cuda.mem_get_info()
        budget = int(0.9 * free)
    pretune(stream, MIXED)
    rep, kept = serve(stream, budget, max_active=args.max_active, chunk=args.chunk, keep_results=(0, 1))
    if args.baseline == "measured":
        pretune(stream, FP64, shared=False)
        base = one_at_a_time_measured(stream)
        drift = compare_finals(rep["finals"], base["finals"])
    else:
        base = one_at_a_time(stream, fp64_step_seconds(sorted({m["nx"] for _, m in stream})))
        drift = None
    check = alone_vs_mix(stream, kept)
    rep.pop("finals")
    base.pop("finals", None)
    out = {"serve_mixed": rep, "one_at_a_time_fp64": base, "speedup_jobs_per_h": rep["jobs_per_h"] / base["jobs_per_h"],
           "mixed_vs_fp64_twin": drift, "alone_vs_mix": check,
           "stream": {"jobs": args.jobs, "rate_per_s": args.rate, "step_scale": args.step_scale,
                      "steps_per_job": [min(m["steps"] for _, m in stream), max(m["steps"] for _, m in stream)],
                      "seed": args.seed, "hbm_budget_gb": budget / 1e9, "fused_planes": args.fused_planes}}
    print(json.dumps(out), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
