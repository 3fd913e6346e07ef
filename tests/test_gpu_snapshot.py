"""Checkpoint and resume of a run's whole time-stepping state
(he4g_save_snapshot / he4g_load_snapshot). The reference restarts from psi,
r and v with three Runge-Kutta-Gill steps (readenc mode 2, DFT4He3d.f90:840);
a snapshot also carries the predictor-corrector history, so a resumed run
continues bit for bit as the saved run, in every arithmetic form, from the
Runge-Kutta start phase and from the predictor-corrector phase."""
import numpy as np
import pytest

from helpers import gpu_run, make_case

pytestmark = pytest.mark.gpu


def _same(a, b, nsteps):
    assert np.array_equal(a.psi, b.psi)
    assert np.array_equal(a.den, b.den)
    assert all(np.array_equal(x, y) for x, y in zip(a.impurity(), b.impurity()))
    assert np.array_equal(a.trajectory()[-nsteps:], b.trajectory())
    assert a.energy() == b.energy()


@pytest.mark.parametrize("precision", [0, 1, 2])
@pytest.mark.parametrize("at", [2, 7])
def test_resume_continues_bit_for_bit(precision, at):
    cfg, tk, psi, r, v, meta = make_case("he100_xe_32", precision=precision)
    a = gpu_run(cfg, tk, psi, r, v)
    a.step(at)
    snap = a.save_snapshot()
    a.step(9)
    # another state in the receiving run, with captured step graphs: the
    # snapshot replaces all of it
    b = gpu_run(cfg, tk, psi * 0.9, r + 0.5, v)
    b.enable_graphs(True)
    b.step(4)
    b.load_snapshot(snap)
    assert b.steps_taken == at
    b.step(9)
    _same(a, b, 9)
    a.close()
    b.close()


@pytest.mark.parametrize("precision", [0, 2])
def test_resume_with_core_otc(precision):
    cfg, tk, psi, r, v, meta = make_case("he100_xe_32", core=1, lsolid=0, hcg=2.190323, precision=precision)
    a = gpu_run(cfg, tk, psi, r, v)
    a.step(5)
    snap = a.save_snapshot()
    b = gpu_run(cfg, tk, psi, r, v)
    b.load_snapshot(snap)
    assert a.energy() == b.energy()  # E_alpha from the restored alpha_s fields
    a.step(6)
    b.step(6)
    _same(a, b, 6)


def test_snapshot_refuses_another_grid_form_or_a_damaged_buffer():
    import he4gpu
    cfg, tk, psi, r, v, meta = make_case("he100_xe_32")
    a = gpu_run(cfg, tk, psi, r, v)
    a.step(4)
    snap = a.save_snapshot()
    c2, tk2, psi2, r2, v2, _ = make_case("he300_ar_48")
    c3, *_ = make_case("he100_xe_32", precision=1)
    for run in (gpu_run(c2, tk2, psi2, r2, v2), gpu_run(c3, tk, psi, r, v)):
        with pytest.raises(he4gpu.He4gError) as e:
            run.load_snapshot(snap)
        assert e.value.code == he4gpu.abi.HE4G_EINVAL
    b = gpu_run(cfg, tk, psi, r, v)
    bad = snap.copy()
    bad[:8] = 0
    for buf in (bad, snap[: snap.size // 2]):
        with pytest.raises(he4gpu.He4gError) as e:
            b.load_snapshot(buf)
        assert e.value.code == he4gpu.abi.HE4G_EINVAL
    # the refused loads left b's own state in place
    b.step(2)
