"""GPU parity at the workloads' own lengths: the FP64 and df64 forms of the
library against the FP64 CPU oracle on the same seeded state.

- The 128^3 He_1000 + Xe collision runs its full 1000 steps (3 RK-Gill +
  997 Hamming predictor-corrector steps, DFT4He3d.f90:834-852), compared
  every 250 steps and, for the impurity, after every step.
- The 256^3 He_5000 + Xe collision runs 3 RK-Gill + 20 predictor-corrector
  steps (the oracle's 2000-step run takes about half an hour of the host's
  cores; tests/records/ holds the longer record).

Tolerance (FP64 build): the density, psi, every energy component, the norm
and the impurity trajectory agree to 1e-10 relative (fields relative to
their maximum, energies relative to max(|E|, 1e-3 K)); the acceleration, a
force sum with cancellation, to 1e-8 of its vector's size.
"""
import numpy as np
import pytest

from helpers import gpu_run, make_case, oracle_run, rel_field, rel_vec

pytestmark = pytest.mark.gpu

TOL = 1e-10
ACC_TOL = 1e-8


def _check_state(g, o, n4, label):
    assert rel_field(g.den, o.den) < TOL, f"{label}: den"
    assert rel_field(g.psi, o.psi) < TOL, f"{label}: psi"
    eg, eo = g.energy(), o.energy()
    for k in eo:
        assert abs(eg[k] - eo[k]) <= TOL * max(abs(eo[k]), 1e-3), f"{label}: {k} {eg[k]} {eo[k]}"
    ng, no = g.observables(n4)["npart"], o.observables(n4)["npart"]
    assert abs(ng - no) <= TOL * abs(no), f"{label}: norm"
    rg, vg, ag = g.impurity()
    ro, vo, ao = o.impurity()
    assert rel_vec(rg, ro) < TOL and rel_vec(vg, vo) < TOL, f"{label}: r/v"
    assert rel_vec(ag, ao) < ACC_TOL, f"{label}: a"


def _oracle_steps(o, k):
    """k oracle steps, one at a time; returns the impurity rows (r, v, a)."""
    rows = []
    for _ in range(k):
        o.step(1)
        r, v, a = o.impurity()
        rows.append(np.concatenate([r, v, a]))
    return np.array(rows)


def _check_trajectory(traj, orows, first_step, label):
    assert traj.shape == (len(orows), 10), label
    assert np.array_equal(traj[:, 0], np.arange(first_step, first_step + len(orows))), label
    for i in range(len(orows)):
        assert rel_vec(traj[i, 1:4], orows[i, 0:3]) < TOL, f"{label}: r at step {first_step + i}"
        assert rel_vec(traj[i, 4:7], orows[i, 3:6]) < TOL, f"{label}: v at step {first_step + i}"
        assert rel_vec(traj[i, 7:10], orows[i, 6:9]) < ACC_TOL, f"{label}: a at step {first_step + i}"


def _run_pair(case, chunks, forms=(0, 2)):
    cfg, tk, psi, r, v, meta = make_case(case)
    o = oracle_run(cfg, tk, psi, r, v)
    runs = {}
    for prec in forms:
        c2, *_ = make_case(case, precision=prec)
        runs[prec] = gpu_run(c2, tk, psi, r, v)
    done = 0
    for k in chunks:
        orows = _oracle_steps(o, k)
        for prec, g in runs.items():
            g.step(k)
            label = f"{case} {'FP64' if prec == 0 else 'df64'} after {done + k} steps"
            _check_trajectory(g.trajectory(), orows, done + 1, label)
            _check_state(g, o, meta["n4"], label)
        done += k
    for g in runs.values():
        g.close()
    o.close()
    return done


def test_config1_full_1000_steps_fp64_and_df64():
    """128^3 He_1000 + Xe: the workload's whole run, 1000 steps."""
    assert _run_pair("he1000_xe_128", [250, 250, 250, 250]) == 1000


def test_config2_256_fp64_and_df64_20_pc_steps():
    """256^3 He_5000 + Xe: 3 RK-Gill + 20 predictor-corrector steps."""
    assert _run_pair("he5000_xe_256", [3, 20]) == 23
