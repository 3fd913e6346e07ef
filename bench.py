#!/usr/bin/env python3
"""Throughput of the time step of the 256^3 He_5000 + Xe collision.

A step is one Hamming predictor–corrector step of psi and the impurity
(steppc.f90) plus the driver's trailing re-evaluation of the impurity
potential, mean field and force (DFT4He3d.f90:849-852): 2 H.psi stencil
sweeps, 2 mean-field evaluations (10 3D FFTs), 2 force reductions. The first
three steps after set_state are Runge–Kutta–Gill steps and fall in the
warm-up. Inputs (psi: 268 MB, history: 1.9 GB) are larger than L2, so no
flush is needed between steps.

The headline line is the FP64 form (the reference's arithmetic). The same
line carries a `mixed` block: the mixed-precision form (FP32 fields, FP64
accumulators and reductions) on the same workload, with its deviation from
the FP64 form after the same steps, and a `df64` block: the FP64 form with its
FFT convolutions in paired-FP32 arithmetic, with the same deviation record.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

N > 1 runs N independent replicas (one per GPU, launched by torchrun); the
path does not shard (every step has global 3D FFTs).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG_DIR = os.path.join(ROOT, "4hetddft-isotropic_gb300")
for _p in (ROOT, PKG_DIR):
    if _p not in sys.path:
        sys.path.insert(0, _p)

CASE = "he5000_xe_256"
METRIC = "steps/s at 256^3 (FP64 predictor-corrector step, He_5000 + Xe)"
PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM = 6800.0
FP64 = 0
MIXED = 1
DF64 = 2
FORM_NAME = {FP64: "FP64", MIXED: "mixed-precision", DF64: "df64"}


def set_case(name):
    global CASE
    CASE = name


def algorithmic_bytes_per_step(nx, ny, nz, prec=FP64, fused_corr=False, fused_xy=False):
    """Compulsory HBM bytes of one predictor-corrector step per kernel family:
    reads + writes of each launch's inputs and outputs, stencil neighbours
    counted once, spectra as (nx/2+1)*ny*nz complex. fused_corr: the inverse
    x pass of the coarse-grained density and the forward x pass of the
    correlation prologue run as one kernel (family fft_x_c2r_corr).
    fused_xy: the y passes run inside the x passes' kernels, one z plane per
    thread-block cluster (families fft_xy_fwd, fft_xy_mid, fft_xy_inv_pot4).
    Returns {family: bytes}."""
    n = nx * ny * nz
    nh = (nx // 2 + 1) * ny * nz
    ev = 2  # potential evaluations per step
    if prec != MIXED:  # FP64 and df64: 8-byte reals, 16-byte complex values
        r, c = 8, 16  # real / complex element
        # R psi 16 pot4 8 uimp 8 timec 4 p3 16 h1 16 h2 16 pc 16 | W p3 16 pc 16 h2 16 den 8
        pred = 156 * n
        # R psit 16 pot4 8 uimp 8 timec 4 p3 16 p2 16 h1 16 h2 16 pc 16 | W pc 16 psi 16 den 8
        corr = 156 * n
    else:
        r, c = 4, 8
        # R psi32 8 pot4 4 uimp 4 timec 4 p3 16 h1 8 h2 8 pc 16 | W p3 16 psi32 8 pc 16 h2 8 den 4
        pred = 120 * n
        # R psit32 8 pot4 4 uimp 4 timec 4 p3 16 p2 16 h1 8 h2 8 pc 16 | W pc 16 psi 16 psi32 8 den 4
        corr = 128 * n
    fam = {
        "pc_predict": pred,
        "pc_correct": corr,
        # FP64: its own pass writing uimp; mixed and df64: uimp is evaluated
        # in the force kernel, whose bytes below include the uimp write
        "potenimp": ev * r * n if prec == FP64 else 0,
        # den -> spectrum; den, dencg -> spectrum (correlation prologue)
        "fft_x_r2c": ev * ((r * n + c * nh) + (2 * r * n + c * nh)),
        # fwd 1, inv 1, fwd 1, inv 1 spectrum: read + write each
        "fft_y": ev * 4 * 2 * c * nh,
        # 1: R spectrum + table | W output + kept forward spectrum; 2: R spectrum + table + kept spectrum +
        # table | W output (the Lennard-Jones product joins the correlation product before the inverse)
        "fft_z_conv": ev * ((c + r + 2 * c) * nh + (c + r + c + r + c) * nh),
        # spectrum -> dencg
        "fft_x_c2r": ev * (c * nh + r * n),
        # spectrum + dencg + den -> pot4
        "fft_x_c2r_pot4": ev * (c * nh + 3 * r * n),
        # FP64: R den + uimp; mixed and df64: R den, W uimp
        "force": ev * 2 * r * n,
        "impurity_scalar": 0,
        "fft_x_c2r_corr": 0,
    }
    if fused_corr or fused_xy:
        # R spectrum, W dencg, R den, W spectrum; the r2c family keeps the plain pass only
        fam["fft_x_c2r_corr"] = ev * (2 * c * nh + 2 * r * n)
        fam["fft_x_c2r"] = 0
        fam["fft_x_r2c"] = ev * (r * n + c * nh)
    if fused_xy:
        # R den | W spectrum; R spectrum, den | W dencg, spectrum; R spectrum, dencg, den | W pot4
        fam["fft_xy_fwd"] = fam.pop("fft_x_r2c")
        fam["fft_xy_mid"] = fam.pop("fft_x_c2r_corr")
        fam["fft_xy_inv_pot4"] = fam.pop("fft_x_c2r_pot4")
        fam["fft_y"] = 0
    return fam


# DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) of each
# kernel family at 256^3, mean over the captured launches; from the ncu
# captures summarised in profiles/fp64_step_he5000_xe_256_kernels.md and
# profiles/mixed_step_he5000_xe_256_kernels.md (FP64 z convolution: the
# capture after the Lennard-Jones product joined the correlation product).
TRAFFIC_256 = {
    FP64: {"potenimp": 71.7e6, "fft_x_r2c": 293.2e6, "fft_y": 216.6e6, "fft_z_conv": 466.8e6,
           "fft_x_c2r": 218.4e6, "fft_x_c2r_pot4": 511.3e6, "force": 268.8e6, "pc_predict": 2581.7e6,
           "pc_correct": 2600.8e6},
    MIXED: {"fft_x_r2c": 126.0e6, "fft_y": 81.5e6, "fft_z_conv": 212.1e6, "fft_x_c2r": 85.9e6,
            "fft_x_c2r_pot4": 244.2e6, "force": 97.1e6, "pc_predict": 1961.1e6, "pc_correct": 2114.0e6},
}


def read_peaks():
    try:
        with open(PEAKS) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-i", str(self.gpu), "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.t.join(timeout=2)

    def summary(self):
        sm, mx = [], []
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 6:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[2:6]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


TILES = None  # fixed FFT tiles (profiling runs) instead of autotuning
CPU_SAMPLE_STEPS = 20  # predictor-corrector steps of the oracle in cpu_baseline (median)


def make_run(prec=FP64, device_tables=False):
    import he4gpu
    psi, r, v, meta = he4gpu.collision_case(CASE)
    kw, tk = he4gpu.config_for_case(meta)
    cfg = he4gpu.default_config(meta["nx"], meta["ny"], meta["nz"], meta["xmax"], precision=prec, **kw)
    run = he4gpu.Run(cfg, selec=tk["selec"], r_cutoff=tk["r_cutoff"], umax=tk["umax"], device_tables=device_tables)
    if TILES:
        run.tiles = TILES
    else:
        run.autotune()
    return run, cfg, psi, r, v, meta


def e2e_measure(run, psi, steps):
    """Steps through the public API with host buffers: per step the impurity
    state goes host->device (he4g_set_impurity, the driver's module variables),
    he4g_step runs one step, and psi plus the impurity state come back to
    pinned host memory (he4g_get_psi_async, he4g_get_impurity). Each step's
    psi copy runs on the library's copy stream while the next step computes;
    the last copy is waited for (he4g_wait_psi) inside the timed region."""
    import numpy as np
    try:
        import torch
        host = torch.empty(psi.size * 2, dtype=torch.float64, pin_memory=True).numpy()
    except Exception:
        host = np.empty(psi.size * 2)
    from he4gpu import abi
    lib, h = run.lib, run.h
    # the first asynchronous read allocates the run's snapshot of psi and its
    # copy stream (set-up, once per run): outside the timed region
    if lib.he4g_get_psi_async(h, abi.dptr(host)) or lib.he4g_wait_psi(h):
        raise RuntimeError("get_psi_async failed")
    rr, vv, aa = run.impurity()
    t0 = time.perf_counter()
    for _ in range(steps):
        run.set_impurity(rr, vv, aa)
        run.step(1)
        # the 72-byte impurity read goes first: issued after the 268 MB psi
        # copy it would queue behind it on the device-to-host copy engine
        rr, vv, aa = run.impurity()
        if lib.he4g_get_psi_async(h, abi.dptr(host)):
            raise RuntimeError("get_psi_async failed")
    if lib.he4g_wait_psi(h):
        raise RuntimeError("wait_psi failed")
    dt = time.perf_counter() - t0
    return steps / dt, 72, psi.size * 16 + 72


def cpu_sample(kind_steps):
    """Times predictor-corrector steps of the FP64 CPU oracle on the workload
    (child process, all host cores). Prints one JSON line with every step's
    time. The process never loads libhe4g.so: the configuration comes from
    he4gpu.reference_config, the Python copy of he4g_default_config."""
    import he4gpu
    from oracle import oracle
    psi, r, v, meta = he4gpu.collision_case(CASE)
    kw, tk = he4gpu.config_for_case(meta)
    cfg = he4gpu.reference_config(meta["nx"], meta["ny"], meta["nz"], meta["xmax"], **kw)
    tabs = oracle.build_tables(cfg, tk["selec"], tk["r_cutoff"], tk["umax"])
    o = oracle.OracleRun(cfg, tabs)
    o.set_state(psi, r, v)
    warm, steps = kind_steps
    # a predictor-corrector step costs the same on any state; the sample skips
    # the Runge–Kutta start and times PC steps plus the trailing evaluation
    for _ in range(warm):
        o.steppc(cfg.deltat)
        o.potenimp(o.impurity()[0])
        o.poten()
        o.forceimp()
    ts = []
    for _ in range(steps):
        t0 = time.perf_counter()
        o.steppc(cfg.deltat)
        o.potenimp(o.impurity()[0])
        o.poten()
        o.forceimp()
        ts.append(time.perf_counter() - t0)
    print(json.dumps({"sec_per_step": statistics.median(ts), "sec_total": sum(ts), "steps": steps, "warmup": warm,
                      "cores": os.cpu_count()}))


def run_cpu_sample(warm, steps):
    env = dict(os.environ)
    env.setdefault("OMP_NUM_THREADS", str(os.cpu_count()))
    r = subprocess.run([sys.executable, os.path.abspath(__file__), "--cpu-sample", str(warm), str(steps), CASE],
                       capture_output=True, text=True, env=env, timeout=1800)
    if r.returncode != 0:
        raise RuntimeError("cpu sample failed: " + r.stderr[-2000:])
    return json.loads(r.stdout.strip().splitlines()[-1])


def dist_env():
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def max_over_ranks(ms, dist, device):
    """The slowest replica's time: the job is done when the last rank is."""
    if dist is None:
        return ms
    import torch
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(ws, steps, ms):
    """Whole-job steps/s: every rank advances its own run by `steps`."""
    return ws * steps / (ms * 1e-3)


def case_grid(case):
    import he4gpu
    c = he4gpu.initial.CASES[case]
    n = c["n"]
    return list(n) if not isinstance(n, int) else [n, n, n]


def metric_name(case, prec=FP64):
    """The headline metric for the 256^3 collision; the same wording with the
    grid and system of any other workload."""
    import he4gpu
    m = METRIC
    if case != "he5000_xe_256":
        c = he4gpu.initial.CASES[case]
        nx, ny, nz = case_grid(case)
        grid = f"{nx}^3" if nx == ny == nz else f"{nx}x{ny}x{nz}"
        m = f"steps/s at {grid} (FP64 predictor-corrector step, He_{c['n4']} + {c['imp']})"
    return m if prec == FP64 else m.replace("FP64", FORM_NAME[prec])


def workload_config(ws, prec=FP64):
    """The `config` object of the JSON line; both arms print the same one."""
    import he4gpu
    c = he4gpu.initial.CASES[CASE]
    grid = case_grid(CASE)
    n = grid[0] * grid[1] * grid[2]
    psi_bytes = 16 * n
    return {"workload": f"{CASE} {FORM_NAME[prec]} predictor-corrector step",
            "grid": grid, "h": c["h"], "n4": c["n4"], "impurity": c["imp"],
            "v_A_per_ps": c["v"], "impact_parameter": f"{c['b_frac']} R",
            "l2": (f"inputs larger than L2 (psi {psi_bytes / 1e6:.0f} MB, history {7 * psi_bytes / 1e9:.2f} GB); "
                   "no flush" if psi_bytes > 129e6 else
                   f"psi {psi_bytes / 1e6:.0f} MB, history {7 * psi_bytes / 1e6:.0f} MB: the step's working set "
                   "exceeds L2; no flush"),
            "parallelism": f"replicas x{ws}"}


def reference_arm(args):
    """The reference's path on the host cores: its Fortran program cannot be
    built (no Fortran compiler, no FFTW/MKL on either machine), so its FP64
    restatement, the oracle, is timed: exactly args.warmup untimed and
    args.steps timed predictor-corrector steps (each with the trailing
    potential and force evaluation) of the same workload as the GPU arm, on
    every host core. The timing process loads liboracle.so only."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    warm = max(0, args.warmup)
    steps = max(1, args.steps)
    s = run_cpu_sample(warm, steps)
    val = steps / s["sec_total"]
    grid = case_grid(CASE)
    line = {
        "impl": "reference", "metric": metric_name(CASE), "value": val, "unit": "steps/s", "n_gpus": args.gpus,
        "steps": steps, "warmup": warm, "ms_per_step": 1e3 * s["sec_total"] / steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded Woods-Saxon droplet + Xe)",
        "config": workload_config(args.gpus),
        "cpu_baseline": {"value": val, "unit": "steps/s", "cores": s["cores"], "kind": "port",
                         "sample": f"{steps} predictor-corrector steps (after {warm} untimed) of the FP64 C oracle "
                                   f"at {'x'.join(map(str, grid))}, OpenMP over {s['cores']} cores; median step "
                                   f"{1e3 * s['sec_per_step']:.1f} ms"},
        "e2e": {"value": val, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def timed_steps(run, cfg, prec, steps, barrier, clock_gpu):
    """Device-timed steps with per-family CUDA-event times and the roofline of
    the dominant family."""
    run.enable_timing(True)
    l0 = run.launch_count
    barrier()
    with ClockSampler(clock_gpu) as clk:
        t_wall = time.perf_counter()
        dev_ms = run.step_timed(steps)
        t_wall = time.perf_counter() - t_wall
    barrier()
    launches = run.launch_count - l0
    fam = run.kernel_times()
    run.enable_timing(False)
    # a repeat without per-launch events gives the step time without their overhead
    barrier()
    dev_ms_clean = run.step_timed(steps)
    barrier()
    ms = min(dev_ms, dev_ms_clean)
    fused = fam.get("fft_x_c2r_corr", (0.0, 0))[1] > 0
    fused_xy = fam.get("fft_xy_mid", (0.0, 0))[1] > 0
    bytes_fam = algorithmic_bytes_per_step(cfg.nx, cfg.ny, cfg.nz, prec, fused, fused_xy)
    tot = sum(v[0] for v in fam.values()) or 1.0
    rows = []
    for name, (fms, nl) in sorted(fam.items(), key=lambda x: -x[1][0]):
        if nl == 0:
            continue
        b = bytes_fam.get(name, 0) * steps
        rows.append({"family": name, "ms_total": round(fms, 4), "launches": nl, "share": round(fms / tot, 4),
                     "gbs": round(b / (fms * 1e-3) / 1e9, 1) if fms > 0 and b else None})
    top = rows[0]
    peak, peak_kind = read_peaks()
    per_launch = bytes_fam[top["family"]] * steps / top["launches"]
    achieved = per_launch / (top["ms_total"] / top["launches"] * 1e-3) / 1e9
    step_bytes = sum(bytes_fam.values())
    step_gbs = step_bytes / (ms / steps * 1e-3) / 1e9
    roofline = {
        "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
        "peak_source": peak_kind, "kernel": top["family"],
        "traffic": (TRAFFIC_256.get(prec, {}).get(top["family"])
                    if (cfg.nx, cfg.ny, cfg.nz) == (256, 256, 256) else None),
        "traffic_source": "ncu dram bytes per launch (profiles/, 256^3 capture)",
        "step_algorithmic_bytes": step_bytes, "step_gbs": step_gbs, "step_frac": step_gbs / peak,
        "families": rows,
    }
    return {"ms": ms, "launches": launches, "clocks": clk.summary(), "wall_s": t_wall, "roofline": roofline}


def ours(args):
    ws, rank, local = dist_env()
    dist = None
    import torch
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist_mod
        dist_mod.init_process_group("nccl")
        dist = dist_mod

    def barrier():
        if dist:
            dist.barrier()
        torch.cuda.synchronize()

    import he4gpu
    he4gpu.abi.load()
    prec = {"fp64": FP64, "mixed": MIXED, "df64": DF64}[args.precision]
    run, cfg, psi, r, v, meta = make_run(prec)
    run.set_state(psi, r, v)
    warm = max(args.warmup, 3)
    run.step(warm)
    res = timed_steps(run, cfg, prec, args.steps, barrier, local)
    ms = max_over_ranks(res["ms"], dist, "cuda")
    value = replica_value(ws, args.steps, ms)
    line = None
    if rank == 0:
        if args.no_e2e:
            e2e_val, h2d, d2h = None, 0, 0
        else:
            e2e_val, h2d, d2h = e2e_measure(run, psi, max(3, min(args.steps, 20)))
        mixed_block = df64_block = None
        if prec == FP64 and ws == 1 and not args.no_mixed:
            mixed_block = form_measure(args, run, barrier, local, MIXED)
        if prec == FP64 and ws == 1 and not args.no_df64:
            df64_block = form_measure(args, run, barrier, local, DF64)
        cufft = None
        if ws == 1 and not args.no_cufft:
            try:
                ours64 = fft_ms_per_evaluation(res["roofline"], args.steps) if prec == FP64 else None
                ours32 = (mixed_block["fft_ms_per_evaluation"] if mixed_block else
                          fft_ms_per_evaluation(res["roofline"], args.steps) if prec == MIXED else None)
                cufft = {"what": "2 r2c + 3 c2r + 3 form-factor products per mean-field evaluation "
                                 "(poten.f90:34-74) through cuFFT (torch.fft), against the library's own "
                                 "FFT passes of one evaluation; comparison only, not on the library's path",
                         "fp64": cufft_compare(cfg.nx, cfg.ny, cfg.nz, ours64, torch.float64),
                         "fp32": cufft_compare(cfg.nx, cfg.ny, cfg.nz, ours32, torch.float32)}
            except Exception as e:  # reported, not fatal
                cufft = {"failed": f"{e}"[:300]}
        cpu = None
        if ws == 1 and not args.no_cpu:
            try:
                s = run_cpu_sample(1, CPU_SAMPLE_STEPS)
                grid = "x".join(map(str, case_grid(CASE)))
                cpu = {"value": 1.0 / s["sec_per_step"], "unit": "steps/s", "cores": s["cores"], "kind": "port",
                       "sample": f"median of {CPU_SAMPLE_STEPS} predictor-corrector steps (after 1 untimed) of "
                                 f"the FP64 C oracle at {grid}, OpenMP over {s['cores']} host cores"}
            except Exception as e:  # reported, not fatal
                cpu = {"value": None, "unit": "steps/s", "cores": os.cpu_count(), "kind": "port",
                       "sample": f"failed: {e}"[:300]}
        rf = res["roofline"]
        line = {
            "metric": metric_name(CASE, prec),
            "value": value, "unit": "steps/s", "n_gpus": ws, "steps": args.steps, "warmup": warm,
            "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": DTYPE[prec],
            "data": "synthetic (seeded Woods-Saxon droplet + Xe)",
            "config": workload_config(ws, prec),
            "fft_tiles": list(run.tiles),
            "grid_point_updates_per_s": value * cfg.nx * cfg.ny * cfg.nz,
            "hbm_gbs": rf["step_gbs"],
            "roofline": rf,
            "fp64_note": ("FP64 issue bounds the FP64 form (GB300: 1.2 TFLOP/s FP64, 1/61 of FP32); ncu shows "
                          "83-85% FP64-pipe activity in every kernel of the step" if prec == FP64 else None),
            "fp64_pipe_busy_ncu": 0.84 if prec == FP64 else None,
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_val * ws if e2e_val else None, "unit": "steps/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "gpu_launches": res["launches"],
            "gpu_launches_per_step": res["launches"] / args.steps,
            "clocks": res["clocks"],
            "wall_s_timed": res["wall_s"],
            "mixed": mixed_block,
            "df64": df64_block,
            "cufft_compare": cufft,
        }
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    run.close()
    if line:
        print(json.dumps(line), flush=True)
    return 0


DTYPE = {
    FP64: "f64",
    MIXED: "mixed (f32 fields, f64 accumulators)",
    DF64: "df64 (paired f32, 48-bit significands: fields, stencils, updates, FFTs, uimp, force; f64 block sums, impurity)",
}
FORM_DTYPE = {
    MIXED: "f32 fields/stencils/FFTs; f64 psi accumulator, reductions, force sum, trajectory",
    DF64: "df64 (paired f32) fields, stencils, updates, FFT convolutions, uimp, force; f64 block sums, trajectory",
}


def form_measure(args, run64, barrier, gpu, prec):
    """Another arithmetic form (mixed or df64) on the same workload, and its
    deviation from the FP64 run after the same number of steps."""
    import numpy as np
    run, cfg, psi, r, v, meta = make_run(prec)
    run.set_state(psi, r, v)
    steps64 = run64.steps_taken
    warm = max(args.warmup, 3)
    run.step(warm)
    res = timed_steps(run, cfg, prec, args.steps, barrier, gpu)
    # bring both runs to the same step count, then compare
    run.step(max(0, steps64 - run.steps_taken))
    extra = run.steps_taken - run64.steps_taken
    if extra > 0:
        run64.step(extra)
    d64, dmx = run64.den, run.den
    e64, emx = run64.energy(), run.energy()
    r64, rmx = run64.impurity()[0], run.impurity()[0]
    dev = {
        "steps": run.steps_taken,
        "den_max_rel": float(np.max(np.abs(dmx - d64)) / np.max(np.abs(d64))),
        "norm_rel": float(abs(dmx.sum() - d64.sum()) / d64.sum()),
        "etot_rel": float(abs(emx["etot"] - e64["etot"]) / abs(e64["etot"])),
        "rimp_abs_A": float(np.max(np.abs(rmx - r64))),
    }
    ms = res["ms"]
    tiles = list(run.tiles)
    run.close()
    rf = res["roofline"]
    return {"value": args.steps / (ms * 1e-3), "unit": "steps/s", "ms_per_step": ms / args.steps,
            "fft_ms_per_evaluation": fft_ms_per_evaluation(rf, args.steps),
            "dtype": FORM_DTYPE[prec],
            "fft_tiles": tiles,
            "hbm_gbs": rf["step_gbs"], "roofline": rf, "gpu_launches": res["launches"],
            "clocks": res["clocks"], "vs_fp64": dev}


def fft_ms_per_evaluation(roofline, steps):
    """Device time of the 3D FFT line passes of one mean-field evaluation
    (two per step), from the per-family CUDA-event times of a timed run. The
    passes include what is fused into them: the correlation prologue, the
    form-factor products and the pot4 epilogue."""
    ms = sum(f["ms_total"] for f in roofline["families"] if f["family"].startswith("fft_"))
    return ms / (2 * steps)


def cufft_compare(nx, ny, nz, ours_ms, real_dtype, reps=20):
    """cuFFT (through torch.fft, timed only as a comparison: it is not on the
    library's path) doing the transforms of one mean-field evaluation of
    poten.f90:34-74 at the workload's grid: r2c of den, the products with the
    coarse-graining and Lennard-Jones form factors and their two c2r, r2c of
    the correlation field, its product and c2r (2 r2c + 3 c2r + 3 products,
    the reference's FFTW sequence). CUDA events on torch's stream, after
    warm-up; the inputs exceed L2 at 256^3. ours_ms: the library's own FFT
    passes per evaluation (fused prologue/epilogue included)."""
    import torch
    dev = torch.device("cuda")
    cdt = torch.complex128 if real_dtype == torch.float64 else torch.complex64
    rb = 8 if real_dtype == torch.float64 else 4
    g = torch.Generator(device=dev)
    g.manual_seed(1)
    shape = (nz, ny, nx)
    den = torch.rand(shape, dtype=real_dtype, device=dev, generator=g)
    corr = torch.rand(shape, dtype=real_dtype, device=dev, generator=g)
    hshape = (nz, ny, nx // 2 + 1)
    wcg = torch.rand(hshape, dtype=real_dtype, device=dev, generator=g)
    vlj = torch.rand(hshape, dtype=real_dtype, device=dev, generator=g)
    S = torch.empty(hshape, dtype=cdt, device=dev)
    T = torch.empty(hshape, dtype=cdt, device=dev)
    out = [torch.empty(shape, dtype=real_dtype, device=dev) for _ in range(3)]

    def evaluation():
        torch.fft.rfftn(den, out=S)
        torch.mul(S, wcg, out=T)
        torch.fft.irfftn(T, s=shape, out=out[0])
        torch.mul(S, vlj, out=T)
        torch.fft.irfftn(T, s=shape, out=out[1])
        torch.fft.rfftn(corr, out=S)
        torch.mul(S, wcg, out=T)
        torch.fft.irfftn(T, s=shape, out=out[2])

    for _ in range(3):
        evaluation()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        evaluation()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    n, nh = nx * ny * nz, (nx // 2 + 1) * ny * nz
    cb = 2 * rb
    # each transform reads its input and writes its output once; each
    # product reads a spectrum and a table and writes a spectrum
    alg = 2 * (rb * n + cb * nh) + 3 * (cb * nh + rb * n) + 3 * (2 * cb * nh + rb * nh)
    peak, kind = read_peaks()
    del den, corr, wcg, vlj, S, T, out
    torch.cuda.empty_cache()
    return {"cufft_ms_per_evaluation": ms, "ours_ms_per_evaluation": ours_ms,
            "ours_speedup_vs_cufft": ms / ours_ms if ours_ms else None,
            "cufft_algorithmic_bytes": alg, "cufft_gbs": alg / (ms * 1e-3) / 1e9,
            "cufft_hbm_frac": alg / (ms * 1e-3) / 1e9 / peak, "peak_source": kind}


def aux_pass(args):
    """Profiling runs only: the kernels off the steady predictor-corrector
    step, once per arithmetic form on the workload's grid: the device set-up
    of the k-space tables, set_state (conversions, density, first
    evaluation), the three Runge-Kutta-Gill steps and two predictor-corrector
    steps, the energies and observables, an asynchronous psi read and (FP64)
    the allocation-free force on caller-owned arrays. Prints one JSON line of
    the forms' energies; times nothing."""
    import numpy as np
    import torch
    torch.cuda.set_device(0)
    out = {}
    for prec in (FP64, MIXED, DF64):
        run, cfg, psi, r, v, meta = make_run(prec, device_tables=True)
        run.set_state(psi, r, v)
        run.step(5)
        e = run.energy()
        run.observables(meta["n4"])
        buf = np.empty(run.shape, dtype=np.complex128)
        run.get_psi_async(buf)
        run.wait_psi()
        if prec == FP64:  # the force on caller-owned arrays, without allocation
            import ctypes
            den = torch.from_numpy(run.den).to("cuda")
            uimp = torch.from_numpy(run.field("uimp")).to("cuda")
            force = torch.empty(3, dtype=torch.float64, device="cuda")
            if run.lib.he4g_forceimp_noalloc(ctypes.c_void_p(den.data_ptr()), ctypes.c_void_p(uimp.data_ptr()),
                                             cfg.nx, cfg.ny, cfg.nz, cfg.xmax, cfg.ymax, cfg.zmax,
                                             ctypes.c_void_p(force.data_ptr()),
                                             ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)):
                raise RuntimeError("he4g_forceimp_noalloc failed")
            torch.cuda.synchronize()
        out[FORM_NAME[prec]] = {"etot": e["etot"], "steps": run.steps_taken}
        run.close()
    print(json.dumps({"aux": out, "workload": CASE}), flush=True)
    return 0


def main():
    if len(sys.argv) >= 2 and sys.argv[1] == "--cpu-sample":
        if len(sys.argv) > 4:
            set_case(sys.argv[4])
        cpu_sample((int(sys.argv[2]), int(sys.argv[3])))
        return 0
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed", "df64"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU-oracle baseline sample")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end pass (profiling runs)")
    ap.add_argument("--no-mixed", action="store_true", help="skip the mixed-precision block")
    ap.add_argument("--no-df64", action="store_true", help="skip the df64 block")
    ap.add_argument("--no-cufft", action="store_true", help="skip the cuFFT comparison")
    ap.add_argument("--case", default=CASE, help="workload (profiling runs use smaller ones)")
    ap.add_argument("--aux", action="store_true",
                    help="profiling runs: set-up, Runge-Kutta, energy and readback kernels of every form, untimed")
    ap.add_argument("--tiles", default=None,
                    help="FFT tiles lpb_r2c,lpb_c2r,log2cols_y,log2cols_z instead of autotuning (profiling runs)")
    args = ap.parse_args()
    set_case(args.case)
    if args.tiles:
        global TILES
        TILES = tuple(int(t) for t in args.tiles.split(","))
    if args.impl == "reference":
        return reference_arm(args)
    if args.aux:
        return aux_pass(args)
    return ours(args)


if __name__ == "__main__":
    sys.exit(main())
