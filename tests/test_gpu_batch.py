"""GPU checks of graph replay and of several runs advancing together.

A captured predictor-corrector step replays the same kernels in the same
order, and runs that share the GPU touch disjoint memory with deterministic
reductions, so both must reproduce direct, one-run-at-a-time stepping bit for
bit: a collision's result is the same alone and in the mix.
"""
import numpy as np
import pytest

from helpers import gpu_run, make_case, rel_field

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [0, 1, 2])
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


@pytest.mark.parametrize("precision", [0, 1, 2])
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


@pytest.mark.parametrize("precision", [0, 1, 2])
def test_batch_graph_matches_runs_alone(precision):
    """he4g_batch_step: all runs' predictor-corrector steps in one graph per
    batch step; 3 Runge-Kutta steps run run by run, then 24 predictor-
    corrector steps cover the 10 arrangements of every run twice. The runs
    start at different phases (one has 2 steps more), so the batch graphs
    key on mixed arrangements. Each run ends bit for bit where it ends alone."""
    import he4gpu
    cases = ["he100_xe_32", "he300_ar_48", "he200_xe_40x48x64"]
    alone, members, pre = [], [], [0, 2, 0]
    for c, k in zip(cases, pre):
        cfg, tk, psi, r, v, meta = make_case(c, precision=precision)
        x = gpu_run(cfg, tk, psi, r, v)
        x.step(27 + k)
        alone.append(x)
        y = gpu_run(cfg, tk, psi, r, v)
        y.enable_graphs(True)
        y.step(k)
        members.append(y)
    b = he4gpu.Batch(members)
    b.step(27)
    assert 1 <= b.graphs <= 10
    for x, y in zip(alone, members):
        assert x.steps_taken == y.steps_taken
        assert np.array_equal(x.psi, y.psi)
        assert all(np.array_equal(p, q) for p, q in zip(x.impurity(), y.impurity()))
        assert np.array_equal(x.trajectory(), y.trajectory())
        assert x.energy() == y.energy()
    # a member run is destroyed: the batch refuses to step and can be freed
    members[1].close()
    with pytest.raises(he4gpu.He4gError) as e:
        b.step(1)
    assert e.value.code == he4gpu.abi.HE4G_ESTATE
    b.close()


@pytest.mark.parametrize("engine", [0, 15])
@pytest.mark.parametrize("precision", [0, 1, 2])
def test_tile_shapes_give_identical_results(precision, engine):
    """Every generic tile shape transforms each line with the same arithmetic:
    three fixed shapes and three drawn at random (seeded) from those that fit."""
    import he4gpu
    cfg, tk, psi, r, v, meta = make_case("he200_xe_40x48x64", precision=precision)
    rng = np.random.default_rng(1000 * precision + engine)
    shapes = [(32, 32, 3, 3), (1, 3, 0, 1), (4, 64, 5, 2)]
    probe = gpu_run(cfg, tk, psi, r, v)
    for _ in range(200):
        if len(shapes) == 6:
            break
        t = (int(2 ** rng.integers(0, 7)), int(rng.integers(1, 65)), int(rng.integers(0, 6)), int(rng.integers(0, 6)))
        try:
            probe.tiles = t + (engine,)
        except he4gpu.He4gError:
            continue  # does not fit in shared memory
        shapes.append(t)
    assert len(shapes) == 6
    probe.close()
    runs = []
    for t in shapes:
        x = gpu_run(cfg, tk, psi, r, v)
        x.tiles = t + (engine,)
        x.enable_graphs(True)
        x.step(8)
        runs.append(x)
    a = runs[0]
    ta = a.trajectory()  # rows since the last read: read each run once
    assert len(ta) == 8
    for x in runs[1:]:
        assert np.array_equal(a.psi, x.psi)
        assert np.array_equal(a.den, x.den)
        assert np.array_equal(ta, x.trajectory())


@pytest.mark.parametrize("case", ["he100_xe_32", "he300_ar_48", "he200_xe_40x48x64"])
@pytest.mark.parametrize("precision", [0, 1, 2])
def test_register_engine_matches_generic(case, precision):
    """The specialised four-step kernels and the generic Stockham kernels
    compute the same transforms; they differ by rounding only."""
    cfg, tk, psi, r, v, meta = make_case(case, precision=precision)
    a = gpu_run(cfg, tk, psi, r, v)
    b = gpu_run(cfg, tk, psi, r, v)
    assert a.tiles[4] == 15  # every length of these grids is specialised
    b.tiles = b.tiles[:4] + (0,)
    a.step(6)
    b.step(6)
    tol = 2e-5 if precision == 1 else 1e-12
    assert rel_field(a.den, b.den) < tol
    assert rel_field(a.field("pot4"), b.field("pot4")) < tol
    assert np.max(np.abs(a.impurity()[0] - b.impurity()[0])) < 1e-9


@pytest.mark.parametrize("case", ["he1000_xe_128", "he5000_xe_256"])
def test_fused_plane_kernels_match_separate_passes(case):
    """The cluster kernels that fuse the y pass with the x passes of each z
    plane (mixed form) transform every line with the register engine's
    arithmetic; they agree with the separate passes to FP32 rounding."""
    cfg, tk, psi, r, v, meta = make_case(case, precision=1)
    a = gpu_run(cfg, tk, psi, r, v)
    b = gpu_run(cfg, tk, psi, r, v)
    assert a.tiles[4] & 16 == 0  # not a default choice
    b.tiles = a.tiles[:4] + (a.tiles[4] | 16,)
    b.enable_timing(True)
    a.step(4)
    b.step(4)
    fams = {k for k, (ms, n) in b.kernel_times().items() if n > 0}
    assert {"fft_xy_fwd", "fft_xy_mid", "fft_xy_inv_pot4"} <= fams
    assert not fams & {"fft_y", "fft_x_c2r_pot4", "fft_x_c2r_corr"}
    assert rel_field(b.den, a.den) < 2e-5
    assert rel_field(b.field("pot4"), a.field("pot4")) < 2e-5
    assert rel_field(b.field("dencg"), a.field("dencg")) < 2e-5
    assert np.max(np.abs(a.impurity()[0] - b.impurity()[0])) < 1e-9


def test_fused_plane_kernels_replay_in_graphs():
    cfg, tk, psi, r, v, meta = make_case("he1000_xe_128", precision=1)
    runs = []
    for graphs in (False, True):
        x = gpu_run(cfg, tk, psi, r, v)
        x.tiles = x.tiles[:4] + (x.tiles[4] | 16,)
        x.enable_graphs(graphs)
        x.step(7)
        runs.append(x)
    assert np.array_equal(runs[0].psi, runs[1].psi)
    assert np.array_equal(runs[0].trajectory(), runs[1].trajectory())


def test_autotune_keeps_a_valid_choice():
    cfg, tk, psi, r, v, meta = make_case("he200_xe_40x48x64", precision=1)
    b = gpu_run(cfg, tk, psi, r, v)
    tuned = b.autotune(reps=2)
    assert b.tiles == tuned
    c = gpu_run(cfg, tk, psi, r, v)
    c.tiles = tuned
    b.step(5)
    c.step(5)
    assert np.array_equal(b.psi, c.psi)


def test_set_tiles_rejects_out_of_range_shapes():
    import he4gpu
    cfg, tk, psi, r, v, meta = make_case("he100_xe_32")
    a = gpu_run(cfg, tk, psi, r, v)
    before = a.tiles
    for bad in [(0, 4, 3, 3, 0), (4, 4, -1, 3, 0), (4, 4, 3, 9, 0), (4, 100, 3, 3, 0), (4, 4, 3, 3, 16),
                (4, 4, 3, 3, 32)]:
        with pytest.raises(he4gpu.He4gError):
            a.tiles = bad
    assert a.tiles == before
