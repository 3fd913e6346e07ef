"""CPU checks of the committed long-run records (tests/records/*.json, written
on a GB300 by tests/records/make_records.py): every recorded deviation meets
the tolerance the record claims.

- parity records: FP64 and df64 GPU forms against the FP64 oracle, and df64
  against FP64, within 1e-10 relative (density and psi relative to their
  maximum, energies relative to max(|E|, 1e-3 K), the norm, r and v of the
  impurity); the acceleration within 1e-8 of its vector's size.
- the mixed-form drift record: after 10^4 steps the total energy within
  1e-6 relative of the FP64 form's and the norm within 1e-8.
"""
import glob
import json
import os

import pytest

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "records")
TOL = 1e-10


def _records(pattern):
    files = sorted(glob.glob(os.path.join(HERE, pattern)))
    if not files:
        pytest.skip(f"no {pattern} record")
    return [(os.path.basename(f), json.load(open(f))) for f in files]


def _within(dev, label):
    for k in ("den_max_rel", "psi_max_rel", "energy_max_rel", "norm_rel", "rimp_rel", "vimp_rel"):
        assert dev[k] < TOL, f"{label}: {k} = {dev[k]}"
    assert dev["aimp_rel"] < 1e-8, f"{label}: aimp_rel = {dev['aimp_rel']}"


def test_parity_records_meet_1e_10():
    for name, rec in _records("parity_*.json"):
        assert rec["checkpoints"][-1]["steps"] == rec["steps"], name
        compared_to_oracle = 0
        for row in rec["checkpoints"]:
            _within(row["df64_vs_fp64"], f"{name} step {row['steps']} df64 vs FP64")
            for key in ("fp64_vs_oracle", "df64_vs_oracle"):
                if key in row:
                    _within(row[key], f"{name} step {row['steps']} {key}")
                    compared_to_oracle += 1
        assert compared_to_oracle >= 2, name
        assert rec["trajectory_df64_vs_fp64_max_rel"] < TOL, name


def test_mixed_drift_record_meets_the_serving_bar():
    for name, rec in _records("drift_mixed_*.json"):
        last = rec["with_absorber"][-1]
        assert last["steps"] == rec["steps"] >= 10000, name
        assert last["dE_rel_mixed_vs_fp64"] < 1e-6, name
        assert last["norm_rel_mixed_vs_fp64"] < 1e-8, name
        off = rec["absorber_off"][-1]
        assert off["norm_rel_mixed_vs_fp64"] < 1e-8, name
