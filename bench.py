#!/usr/bin/env python3
"""Throughput of the FP64 time step of the 256^3 He_5000 + Xe collision.

A step is one Hamming predictor–corrector step of psi and the impurity
(steppc.f90) plus the driver's trailing re-evaluation of the impurity
potential, mean field and force (DFT4He3d.f90:849-852): 2 H.psi stencil
sweeps, 2 mean-field evaluations (10 3D FFTs), 2 force reductions. The first
three steps after set_state are Runge–Kutta–Gill steps and fall in the
warm-up. Inputs (psi: 268 MB, history: 1.9 GB) are larger than L2, so no
flush is needed between steps.

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


def set_case(name):
    global CASE
    CASE = name


def algorithmic_bytes_per_step(nx, ny, nz):
    """Compulsory HBM bytes of one predictor-corrector step per kernel family
    (reads + writes of each launch's inputs and outputs, stencil neighbours
    counted once, spectra as (nx/2+1)*ny*nz complex). Returns {family: bytes}."""
    n = nx * ny * nz
    nh = (nx // 2 + 1) * ny * nz
    ev = 2  # potential evaluations per step
    return {
        # R psi 16 pot4 8 uimp 8 timec 4 p3 16 h1 16 h2 16 pc 16 | W p3 16 pc 16 h2 16 den 8
        "pc_predict": 156 * n,
        # R psit 16 pot4 8 uimp 8 timec 4 p3 16 p2 16 h1 16 h2 16 pc 16 | W pc 16 psi 16 den 8
        "pc_correct": 156 * n,
        "potenimp": ev * 8 * n,
        # den -> spec (8 + 16 nh/n), den,dencg -> spec (16 + 16 nh/n)
        "fft_x_r2c": ev * (8 * n + 16 * nh + 16 * n + 16 * nh),
        # 4 launches: fwd 1 spectrum, inv 2 spectra, fwd 1, inv 1 (read + write each)
        "fft_y": ev * (32 * nh + 64 * nh + 32 * nh + 32 * nh),
        # conv 1: R 16 + 2 tables x 8 | W 2 x 16 ; conv 2: R 16 + 8 | W 16
        "fft_z_conv": ev * (64 * nh + 40 * nh),
        # 2 spectra -> dencg, delj4
        "fft_x_c2r": ev * (32 * nh + 16 * n),
        # conv spectrum + delj4, dencg, den -> pot4
        "fft_x_c2r_pot4": ev * (16 * nh + 32 * n),
        # R den 8 + uimp 8
        "force": ev * 16 * n,
        "impurity_scalar": 0,
    }


def launches_per_step():
    # per evaluation: potenimp 1, r2c 2, y 4, zconv 2, c2r 1, pot4 1, force 1, scalar 1 = 13
    return 2 + 2 + 2 * 13


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


def make_run():
    import he4gpu
    psi, r, v, meta = he4gpu.collision_case(CASE)
    kw, tk = he4gpu.config_for_case(meta)
    cfg = he4gpu.default_config(meta["nx"], meta["ny"], meta["nz"], meta["xmax"], **kw)
    run = he4gpu.Run(cfg, selec=tk["selec"], r_cutoff=tk["r_cutoff"], umax=tk["umax"])
    return run, cfg, psi, r, v, meta


def e2e_measure(run, psi, r, v, steps):
    """Steps through the public API with host buffers: per step the impurity
    state goes host->device (he4g_set_impurity, the driver's module variables),
    he4g_step runs one step, and psi plus the impurity state come back to
    pinned host memory (he4g_get_psi, he4g_get_impurity)."""
    import numpy as np
    try:
        import torch
        host = torch.empty(psi.size * 2, dtype=torch.float64, pin_memory=True).numpy()
    except Exception:
        host = np.empty(psi.size * 2)
    from he4gpu import abi
    lib, h = run.lib, run.h
    rr, vv, aa = run.impurity()
    t0 = time.perf_counter()
    for _ in range(steps):
        run.set_impurity(rr, vv, aa)
        run.step(1)
        rc = lib.he4g_get_psi(h, abi.dptr(host))
        if rc:
            raise RuntimeError("get_psi failed")
        rr, vv, aa = run.impurity()
    dt = time.perf_counter() - t0
    h2d = 72
    d2h = psi.size * 16 + 72
    return steps / dt, h2d, d2h


def cpu_sample(kind_steps):
    """Times predictor-corrector steps of the FP64 CPU oracle at 256^3 (child
    process, all host cores). Prints one JSON line."""
    import numpy as np

    import he4gpu
    from oracle import oracle
    psi, r, v, meta = he4gpu.collision_case(CASE)
    kw, tk = he4gpu.config_for_case(meta)
    cfg = he4gpu.default_config(meta["nx"], meta["ny"], meta["nz"], meta["xmax"], **kw)
    tabs = oracle.build_tables(cfg, tk["selec"], tk["r_cutoff"], tk["umax"])
    o = oracle.OracleRun(cfg, tabs)
    o.set_state(psi, r, v)
    warm, steps = kind_steps
    # the predictor-corrector step costs the same on any state; the sample
    # skips the Runge–Kutta start and times PC steps directly
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
    del np
    print(json.dumps({"sec_per_step": statistics.median(ts), "steps": steps, "cores": os.cpu_count()}))


def run_cpu_sample(warm, steps):
    env = dict(os.environ)
    env.setdefault("OMP_NUM_THREADS", str(os.cpu_count()))
    r = subprocess.run([sys.executable, os.path.abspath(__file__), "--cpu-sample", str(warm), str(steps)],
                       capture_output=True, text=True, env=env, timeout=1800)
    if r.returncode != 0:
        raise RuntimeError("cpu sample failed: " + r.stderr[-2000:])
    return json.loads(r.stdout.strip().splitlines()[-1])


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def reference_arm(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    # the reference's own Fortran program cannot be built (no Fortran compiler,
    # no FFTW); its restatement (the FP64 oracle) is timed instead
    warm = max(0, min(args.warmup, 2))
    steps = max(1, min(args.steps, 8))
    s = run_cpu_sample(warm, steps)
    val = 1.0 / s["sec_per_step"]
    line = {
        "impl": "reference", "metric": METRIC, "value": val, "unit": "steps/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * s["sec_per_step"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded Woods-Saxon droplet + Xe)",
        "config": {"workload": CASE, "grid": [256, 256, 256], "h": 0.4, "n4": 5000, "impurity": "Xe",
                   "steps_timed": steps},
        "cpu_baseline": {"value": val, "unit": "steps/s", "cores": s["cores"], "kind": "port",
                         "sample": f"{steps} predictor-corrector steps of the FP64 C oracle at 256^3 "
                                   f"(median), OpenMP over {s['cores']} cores"},
        "e2e": {"value": val, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def ours(args):
    import numpy as np
    ws, rank, local = dist_env()
    dist = None
    if ws > 1:
        import torch
        import torch.distributed as dist_mod
        torch.cuda.set_device(local)
        dist_mod.init_process_group("nccl")
        dist = dist_mod
    else:
        try:
            import torch
            torch.cuda.set_device(0)
        except Exception:
            pass
    import he4gpu
    he4gpu.abi.load()
    run, cfg, psi, r, v, meta = make_run()
    run.set_state(psi, r, v)
    warm = max(args.warmup, 3)
    run.step(warm)

    def barrier():
        if dist:
            dist.barrier()
        try:
            import torch
            torch.cuda.synchronize()
        except Exception:
            pass

    # timed region: K predictor-corrector steps, device-timed on the run's stream
    run.enable_timing(True)
    l0 = run.launch_count
    barrier()
    with ClockSampler(local) as clk:
        t_wall = time.perf_counter()
        dev_ms = run.step_timed(args.steps)
        t_wall = time.perf_counter() - t_wall
    barrier()
    launches = run.launch_count - l0
    fam = run.kernel_times()
    run.enable_timing(False)
    # an untimed-instrumentation repeat gives the step time without event overhead
    barrier()
    dev_ms_clean = run.step_timed(args.steps)
    barrier()
    ms = min(dev_ms, dev_ms_clean)
    if dist:
        import torch
        t = torch.tensor([ms], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = ws * args.steps / (ms * 1e-3)

    # roofline of the dominant kernel family (largest share of device time)
    bytes_fam = algorithmic_bytes_per_step(cfg.nx, cfg.ny, cfg.nz)
    tot = sum(v[0] for v in fam.values()) or 1.0
    fam_rows = []
    for name, (fms, nl) in sorted(fam.items(), key=lambda x: -x[1][0]):
        if nl == 0:
            continue
        b = bytes_fam.get(name, 0) * args.steps
        fam_rows.append({"family": name, "ms_total": fms, "launches": nl, "share": fms / tot,
                         "gbs": (b / (fms * 1e-3) / 1e9) if fms > 0 and b else None})
    top = fam_rows[0]
    peak, peak_kind = read_peaks()
    per_launch_bytes = bytes_fam[top["family"]] * args.steps / top["launches"]
    achieved = per_launch_bytes / (top["ms_total"] / top["launches"] * 1e-3) / 1e9
    step_bytes = sum(bytes_fam.values())
    roofline = {
        "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
        "peak_source": peak_kind, "kernel": top["family"], "traffic": None,
        "step_algorithmic_bytes": step_bytes,
        "step_gbs": step_bytes / (ms / args.steps * 1e-3) / 1e9,
        "step_frac": step_bytes / (ms / args.steps * 1e-3) / 1e9 / peak,
        "families": fam_rows,
        "note": "FP64 issue rate (1.2 TFLOP/s measured on this GPU) bounds this path, not HBM",
    }
    line = None
    if rank == 0:
        e2e_steps = max(3, min(args.steps, 10))
        if args.no_e2e:
            e2e_val, h2d, d2h = None, 0, 0
        else:
            e2e_val, h2d, d2h = e2e_measure(run, psi, r, v, e2e_steps)
        cpu = None
        if ws == 1 and not args.no_cpu:
            try:
                s = run_cpu_sample(1, 2)
                cpu = {"value": 1.0 / s["sec_per_step"], "unit": "steps/s", "cores": s["cores"], "kind": "port",
                       "sample": "2 predictor-corrector steps of the FP64 C oracle at 256^3 (median of 2, after 1 "
                                 "warm-up), OpenMP over all host cores"}
            except Exception as e:  # reported, not fatal
                cpu = {"value": None, "unit": "steps/s", "cores": os.cpu_count(), "kind": "port",
                       "sample": f"failed: {e}"[:300]}
        line = {
            "metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": ws, "steps": args.steps,
            "warmup": warm, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded Woods-Saxon droplet + Xe)",
            "config": {"workload": CASE + " FP64 predictor-corrector step", "grid": [cfg.nx, cfg.ny, cfg.nz],
                       "h": meta["h"], "n4": meta["n4"], "impurity": meta["imp"], "v_A_per_ps": meta["v"],
                       "impact_parameter": f"{meta['b_frac']} R",
                       "l2": "inputs larger than L2 (psi 268 MB, history 1.9 GB); no flush",
                       "parallelism": f"replicas x{ws}"},
            "grid_point_updates_per_s": value * cfg.nx * cfg.ny * cfg.nz,
            "hbm_gbs": roofline["step_gbs"],
            "roofline": roofline,
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_val * ws if e2e_val else None, "unit": "steps/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "gpu_launches": launches,
            "gpu_launches_per_step": launches / args.steps,
            "clocks": clk.summary(),
            "wall_s_timed": t_wall,
        }
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    run.close()
    if line:
        print(json.dumps(line), flush=True)
    del np
    return 0


def main():
    if len(sys.argv) >= 2 and sys.argv[1] == "--cpu-sample":
        cpu_sample((int(sys.argv[2]), int(sys.argv[3])))
        return 0
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU-oracle baseline sample")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end pass (profiling runs)")
    ap.add_argument("--case", default=CASE, help="workload (profiling runs use smaller ones)")
    args = ap.parse_args()
    set_case(args.case)
    if args.impl == "reference":
        return reference_arm(args)
    return ours(args)


if __name__ == "__main__":
    sys.exit(main())
