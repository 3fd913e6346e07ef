"""Drift of the mixed-precision (or df64) form against the FP64 form over a
long run.

Runs one collision case twice on the GPU, in FP64 (the reference's
arithmetic, checked against the CPU oracle to 1e-10 by the parity tests) and
in the other form, for the same number of steps, and reports at checkpoints
the relative total-energy difference |E_form - E_fp64| / |E_fp64|, the
relative norm difference, the maximum density difference relative to
max(den), and the impurity-position difference in Angstrom. It also reports
each form's own drift from its initial energy and norm.

  python -m he4gpu.drift --case he5000_xe_256 --steps 10000 --every 1000
  python -m he4gpu.drift --form df64 --steps 2000 --every 500
"""
import argparse
import json
import sys
import time

import numpy as np

from . import collision_case, config_for_case, default_config, Run


def run_case(case, precision, steps, every, absorber=True):
    psi, r, v, meta = collision_case(case)
    kw, tk = config_for_case(meta)
    if not absorber:
        kw["lambdah"] = 0.0
    cfg = default_config(meta["nx"], meta["ny"], meta["nz"], meta["xmax"], meta["ymax"], meta["zmax"],
                         precision=precision, **kw)
    run = Run(cfg, selec=tk["selec"], r_cutoff=tk["r_cutoff"], umax=tk["umax"])
    run.set_state(psi, r, v)
    return run, meta


FORMS = {"mixed": 1, "df64": 2}


def compare(case, steps, every, absorber=True, form="mixed"):
    a, meta = run_case(case, 0, steps, every, absorber)
    b, _ = run_case(case, FORMS[form], steps, every, absorber)
    n4 = meta["n4"]
    e0a, e0b = a.energy()["etot"], b.energy()["etot"]
    n0a, n0b = a.observables(n4)["npart"], b.observables(n4)["npart"]
    rows = []
    done = 0
    t0 = time.time()
    while done < steps:
        k = min(every, steps - done)
        a.step(k)
        b.step(k)
        done += k
        ea, eb = a.energy()["etot"], b.energy()["etot"]
        na, nb = a.observables(n4)["npart"], b.observables(n4)["npart"]
        da, db = a.den, b.den
        ra, rb = a.impurity()[0], b.impurity()[0]
        rows.append({
            "steps": done,
            "etot_fp64": ea, f"etot_{form}": eb,
            f"dE_rel_{form}_vs_fp64": abs(eb - ea) / abs(ea),
            f"norm_rel_{form}_vs_fp64": abs(nb - na) / na,
            f"den_max_rel_{form}_vs_fp64": float(np.max(np.abs(db - da)) / np.max(np.abs(da))),
            "rimp_diff_A": float(np.max(np.abs(rb - ra))),
            "rimp_rel": float(np.max(np.abs(rb - ra)) / np.max(np.abs(ra))),
            "dE_rel_fp64_vs_start": abs(ea - e0a) / abs(e0a),
            f"dE_rel_{form}_vs_start": abs(eb - e0b) / abs(e0b),
            "norm_rel_fp64_vs_start": abs(na - n0a) / n0a,
            f"norm_rel_{form}_vs_start": abs(nb - n0b) / n0b,
            "wall_s": time.time() - t0,
        })
        print(json.dumps(rows[-1]), flush=True)
    a.close()
    b.close()
    return rows


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--case", default="he5000_xe_256")
    ap.add_argument("--steps", type=int, default=10000)
    ap.add_argument("--every", type=int, default=1000)
    ap.add_argument("--no-absorber", action="store_true")
    ap.add_argument("--form", default="mixed", choices=sorted(FORMS))
    args = ap.parse_args(argv)
    compare(args.case, args.steps, args.every, absorber=not args.no_absorber, form=args.form)
    return 0


if __name__ == "__main__":
    sys.exit(main())
