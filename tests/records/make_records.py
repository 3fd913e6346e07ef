"""Writes the long-run parity and drift records of the collision workloads.

Test infrastructure: it drives the GPU library through its C ABI and the FP64
CPU oracle, and writes JSON files beside itself that tests/test_records.py
checks against the stated tolerances. It needs a GPU.

  python tests/records/make_records.py parity_256   # 256^3: FP64 and df64 GPU forms, 2000 steps
  python tests/records/make_records.py drift_mixed  # 256^3: mixed form vs FP64, 10^4 steps
  python tests/records/make_records.py parity_128   # 128^3: both GPU forms and the oracle, 1000 steps

* parity_he5000_xe_256.json: the 256^3 He_5000 + Xe collision run for its
  2000 steps in the FP64 and df64 forms. The oracle runs beside them for the
  first `--oracle-steps` steps (its 2000 steps would take about half an hour
  of the host's cores), so the record holds FP64 GPU vs oracle and df64 GPU
  vs oracle at those checkpoints, and df64 GPU vs FP64 GPU at every
  checkpoint to 2000.
* drift_mixed_he5000_xe_256.json: the mixed-precision form against the FP64
  form over 10^4 steps (1 ps), with the absorber of the shipped input and
  without it (the run's own energy and norm drift), from he4gpu.drift.
* parity_he1000_xe_128.json: the 128^3 He_1000 + Xe collision, 1000 steps,
  both GPU forms against the oracle every 100 steps.
"""
import argparse
import json
import os
import platform
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (ROOT, os.path.join(ROOT, "4hetddft-isotropic_gb300"), os.path.dirname(HERE)):
    if p not in sys.path:
        sys.path.insert(0, p)

FORM = {0: "fp64", 1: "mixed", 2: "df64"}


def _gpu_name():
    try:
        import torch
        return torch.cuda.get_device_name(0)
    except Exception:
        return None


def _state(run, n4):
    e = run.energy()
    r, v, a = run.impurity()
    return {"den": run.den, "psi": run.psi, "energy": e, "norm": run.observables(n4)["npart"], "r": r, "v": v,
            "a": a}


def _compare(a, b):
    """Deviation of state a from state b: fields relative to b's maximum,
    energies relative to max(|E_b|, 1e-3 K), vectors relative to b's size."""
    def vec(x, y):
        return float(np.max(np.abs(x - y)) / max(np.max(np.abs(y)), 1e-300))
    return {
        "den_max_rel": vec(a["den"], b["den"]),
        "psi_max_rel": vec(a["psi"], b["psi"]),
        "energy_max_rel": max(abs(a["energy"][k] - b["energy"][k]) / max(abs(b["energy"][k]), 1e-3)
                              for k in b["energy"]),
        "etot_rel": abs(a["energy"]["etot"] - b["energy"]["etot"]) / abs(b["energy"]["etot"]),
        "norm_rel": abs(a["norm"] - b["norm"]) / abs(b["norm"]),
        "rimp_rel": vec(a["r"], b["r"]),
        "vimp_rel": vec(a["v"], b["v"]),
        "aimp_rel": vec(a["a"], b["a"]),
    }


def parity(case, steps, every, oracle_steps, out_name):
    from helpers import gpu_run, make_case, oracle_run
    cfg, tk, psi, r, v, meta = make_case(case)
    runs = {}
    for prec in (0, 2):
        c, *_ = make_case(case, precision=prec)
        runs[prec] = gpu_run(c, tk, psi, r, v)
    o = oracle_run(cfg, tk, psi, r, v) if oracle_steps else None
    rows = []
    marks = sorted(set(list(range(every, steps + 1, every)) + [m for m in (3, 23) if m <= oracle_steps]
                       + ([oracle_steps] if oracle_steps else [])))
    done, t0 = 0, time.time()
    traj = {p: [] for p in runs}
    for m in marks:
        k = m - done
        for g in runs.values():
            g.step(k)
        for p, g in runs.items():
            traj[p].append(g.trajectory())
        row = {"steps": m}
        st = {p: _state(g, meta["n4"]) for p, g in runs.items()}
        row["df64_vs_fp64"] = _compare(st[2], st[0])
        if o is not None and m <= oracle_steps:
            o.step(k)
            so = _state(o, meta["n4"])
            row["fp64_vs_oracle"] = _compare(st[0], so)
            row["df64_vs_oracle"] = _compare(st[2], so)
        row["etot_fp64"] = st[0]["energy"]["etot"]
        row["norm_fp64"] = st[0]["norm"]
        row["wall_s"] = round(time.time() - t0, 1)
        rows.append(row)
        print(json.dumps(row), flush=True)
        done = m
    if o is not None:
        o.close()
    # impurity trajectories of the two forms, step by step over the whole run
    t64, tdf = np.concatenate(traj[0]), np.concatenate(traj[2])
    rdev = float(np.max(np.abs(tdf[:, 1:4] - t64[:, 1:4]) / np.max(np.abs(t64[:, 1:4]), axis=1, keepdims=True)))
    for g in runs.values():
        g.close()
    rec = {"workload": case, "grid": [meta["nx"], meta["ny"], meta["nz"]], "n4": meta["n4"], "impurity": meta["imp"],
           "steps": steps, "oracle_steps": oracle_steps, "gpu": _gpu_name(), "host": platform.machine(),
           "cores": os.cpu_count(), "tolerance": 1e-10,
           "trajectory_df64_vs_fp64_max_rel": rdev, "checkpoints": rows,
           "made_by": "python tests/records/make_records.py " + out_name}
    with open(os.path.join(HERE, f"parity_{case}.json"), "w") as f:
        json.dump(rec, f, indent=1)


def drift_mixed(case, steps, every):
    from he4gpu import drift
    rec = {"workload": case, "steps": steps, "gpu": _gpu_name(),
           "made_by": "python tests/records/make_records.py drift_mixed"}
    rec["with_absorber"] = drift.compare(case, steps, every, absorber=True, form="mixed")
    rec["absorber_off"] = drift.compare(case, steps, every, absorber=False, form="mixed")
    with open(os.path.join(HERE, f"drift_mixed_{case}.json"), "w") as f:
        json.dump(rec, f, indent=1)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("what", choices=["parity_256", "drift_mixed", "parity_128"])
    ap.add_argument("--oracle-steps", type=int, default=53)
    ap.add_argument("--steps", type=int, default=None)
    a = ap.parse_args()
    import he4gpu
    he4gpu.abi.load()
    if a.what == "parity_256":
        parity("he5000_xe_256", a.steps or 2000, 250, a.oracle_steps, "parity_256")
    elif a.what == "parity_128":
        parity("he1000_xe_128", a.steps or 1000, 100, a.steps or 1000, "parity_128")
    else:
        drift_mixed("he5000_xe_256", a.steps or 10000, 1000)
    return 0


if __name__ == "__main__":
    sys.exit(main())
