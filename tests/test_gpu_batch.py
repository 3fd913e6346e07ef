"""GPU checks of graph replay and of several runs advancing together.

A captured predictor-corrector step replays the same kernels in the same
order, and runs that share the GPU touch disjoint memory with deterministic
reductions, so both must reproduce direct, one-run-at-a-time stepping bit for
bit: a collision's result is the same alone and in the mix.
"""
import numpy as np
import pytest

from helpers import gpu_run, make_case

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [0, 1])
def test_graph_replay_matches_direct_launches(precision):
    cfg, tk, psi, r, v, meta = make_case("he100_xe_32", precision=precision)
    a = gpu_run(cfg, tk, psi, r, v)
    b = gpu_run(cfg, tk, psi, r, v)
    b.enable_graphs(True)
    a.step(27)  # 3 RK + 24 PC steps: every one of the 10 slot arrangements, twice
    b.step(27)
    assert np.array_equal(a.psi, b.psi)
    assert np.array_equal(a.den, b.den)
    ta, tb = a.trajectory(), b.trajectory()
    assert np.array_equal(ta, tb)
    assert a.launch_count == b.launch_count


@pytest.mark.parametrize("precision", [0, 1])
def test_runs_in_the_mix_match_runs_alone(precision):
    import he4gpu
    cases = ["he100_xe_32", "he300_ar_48", "he200_xe_40x48x64"]
    alone, mixed = [], []
    for c in cases:
        cfg, tk, psi, r, v, meta = make_case(c, precision=precision)
        x = gpu_run(cfg, tk, psi, r, v)
        x.step(14)
        alone.append(x)
        y = gpu_run(cfg, tk, psi, r, v)
        y.enable_graphs(True)
        mixed.append(y)
    he4gpu.step_many(mixed, 14)
    for x, y in zip(alone, mixed):
        assert np.array_equal(x.psi, y.psi)
        assert all(np.array_equal(p, q) for p, q in zip(x.impurity(), y.impurity()))
        assert x.energy() == y.energy()


@pytest.mark.parametrize("precision", [0, 1])
def test_autotuned_tiles_give_identical_results(precision):
    """Every tile shape transforms each line with the same arithmetic."""
    cfg, tk, psi, r, v, meta = make_case("he200_xe_40x48x64", precision=precision)
    a = gpu_run(cfg, tk, psi, r, v)
    default = a.tiles
    b = gpu_run(cfg, tk, psi, r, v)
    tuned = b.autotune(reps=2)
    assert b.tiles == tuned
    # force a shape different from the default in every pass
    c = gpu_run(cfg, tk, psi, r, v)
    c.tiles = (1 if default[0] != 1 else 2, 3 if default[1] != 3 else 4,
               0 if default[2] != 0 else 1, 1 if default[3] != 1 else 2)
    for x in (a, b, c):
        x.enable_graphs(True)
        x.step(8)
    ta = a.trajectory()  # rows since the last read: read each run once
    assert len(ta) == 8
    for x in (b, c):
        assert np.array_equal(a.psi, x.psi)
        assert np.array_equal(a.den, x.den)
        assert np.array_equal(ta, x.trajectory())


def test_set_tiles_rejects_out_of_range_shapes():
    import he4gpu
    cfg, tk, psi, r, v, meta = make_case("he100_xe_32")
    a = gpu_run(cfg, tk, psi, r, v)
    before = a.tiles
    for bad in [(0, 4, 3, 3), (4, 4, -1, 3), (4, 4, 3, 9), (4, 100, 3, 3)]:
        with pytest.raises(he4gpu.He4gError):
            a.tiles = bad
    assert a.tiles == before
