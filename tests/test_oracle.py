"""CPU checks of the FP64 oracle against the reference's own data and against
independent implementations (numpy FFT, scipy sine integral)."""
import json
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def small_cfg(nx, ny, nz, xmax=6.0, **kw):
    import he4gpu
    return he4gpu.default_config(nx, ny, nz, xmax, **kw)


@pytest.fixture(scope="module")
def stencil_golden():
    return json.load(open(os.path.join(GOLDEN, "stencil_rows.json")))


@pytest.mark.parametrize("id_", [1, 2])
def test_stencil_rows_equal_blockds(oracle_mod, stencil_golden, id_):
    """The 13-point rows equal the Bickley table rows (blockds.f) bit for bit."""
    import ctypes as C
    rows = (C.c_double * 13)()
    oracle_mod.load().orc_stencil_rows(id_, rows)
    gold = stencil_golden["d%d" % id_]["centre_row"]
    assert list(rows) == gold


@pytest.mark.parametrize("id_", [1, 2])
def test_icon13_is_zero_padding(oracle_mod, stencil_golden, he4gpu_mod, id_):
    """Applying the reference's icon=13 matrix rows to a 13-point grid line gives
    the oracle's zero-padded centred derivative."""
    mat = np.array(stencil_golden["d%d" % id_]["matrix_icon13"])
    cfg = small_cfg(16, 16, 16, xmax=4.0)
    tabs = oracle_mod.build_tables(cfg)
    o = oracle_mod.OracleRun(cfg, tabs)
    rng = np.random.default_rng(3)
    f = rng.normal(size=(16, 16, 16))
    h = 2 * 4.0 / 16
    for axis in range(3):
        d = o.deriv(id_, axis, f)
        line = np.moveaxis(f, 2 - axis, -1)[3, 5]
        dl = np.moveaxis(d, 2 - axis, -1)[3, 5]
        # first/last 13 points use rows 1..13 of the matrix on f(1:13) / f(n-12:n)
        sc = (1.0 / h ** id_)
        first = np.array([np.sum((mat[i] * sc) * line[:13]) for i in range(6)])
        last = np.array([np.sum((mat[i] * sc) * line[-13:]) for i in range(7, 13)])
        np.testing.assert_allclose(dl[:6], first, rtol=1e-13, atol=1e-12)
        np.testing.assert_allclose(dl[-6:], last, rtol=1e-13, atol=1e-12)


def test_derivative_of_polynomial(oracle_mod, he4gpu_mod):
    """13-point rows are exact for polynomials of degree <= 12 away from the edges."""
    cfg = small_cfg(32, 32, 32, xmax=3.2)
    o = oracle_mod.OracleRun(cfg, oracle_mod.build_tables(cfg))
    h = 0.2
    x = -3.2 + h * np.arange(32)
    f = np.broadcast_to((x ** 5 - 2 * x ** 3)[None, None, :], (32, 32, 32)).copy()
    d1 = o.deriv(1, 0, f)[0, 0, 6:-6]
    d2 = o.deriv(2, 0, f)[0, 0, 6:-6]
    xi = x[6:-6]
    np.testing.assert_allclose(d1, 5 * xi ** 4 - 6 * xi ** 2, rtol=1e-10, atol=1e-9)
    np.testing.assert_allclose(d2, 20 * xi ** 3 - 12 * xi, rtol=1e-10, atol=1e-9)


@pytest.mark.parametrize("shape", [(16, 16, 16), (12, 10, 20), (30, 18, 16), (40, 48, 36), (50, 24, 30)])
def test_fft_matches_numpy(oracle_mod, he4gpu_mod, shape):
    """Unnormalised r2c and c2r (fft.f90 conventions) against numpy."""
    nz, ny, nx = shape
    import he4gpu
    cfg = he4gpu.Config()
    cfg.nx, cfg.ny, cfg.nz = nx, ny, nz
    cfg.xmax = cfg.ymax = cfg.zmax = 5.0
    cfg.npot = 11
    cfg.delinter = 2.0
    cfg.hcg = cfg.h4 = 2.19
    cfg.sigma4, cfg.eps4, cfg.l_alpha = 2.556, 10.22, 1.0
    cfg.lambdah, cfg.txmean, cfg.tymean, cfg.tzmean = 2.0, 1000.0, 1000.0, 1000.0
    cfg.txsurf = cfg.tysurf = cfg.tzsurf = 2.0
    o = oracle_mod.OracleRun(cfg, oracle_mod.build_tables(cfg))
    rng = np.random.default_rng(1)
    a = rng.normal(size=shape)
    s = o.r2c(a)
    ref = np.fft.rfftn(a)
    assert np.max(np.abs(s - ref)) < 1e-12 * np.max(np.abs(ref))
    back = o.c2r(s)
    np.testing.assert_allclose(back / a.size, a, rtol=0, atol=1e-13)


def test_sine_integral_matches_scipy(oracle_mod):
    sp = pytest.importorskip("scipy.special")
    lib = oracle_mod.load()
    xs = np.concatenate([np.linspace(1e-6, 3, 301), np.linspace(3, 60, 571), [2.999999, 3.0, 3.000001]])
    got = np.array([lib.orc_si(float(x)) for x in xs])
    ref = sp.sici(xs)[0]
    np.testing.assert_allclose(got, ref, rtol=2e-15, atol=2e-15)


def test_reference_kats(oracle_mod):
    """Known answers quoted in the reference source (tests/golden/reference_kats.json)."""
    lib = oracle_mod.load()
    kats = json.load(open(os.path.join(GOLDEN, "reference_kats.json")))
    got = {
        "V_Xe_He(2.0)": lib.orc_v_xe_he(2.0),
        "V_Ar_He(2.0)": lib.orc_v_ar_he(2.0),
        "V_Xe_He(2.55)": lib.orc_v_xe_he(2.55),
        "bforce_OT(eps4=10.22, sigma4=2.556, h4ot=2.190323)": lib.orc_bforce(10.22, 2.556, 2.190323),
    }
    for k in kats:
        v = got[k["what"]]
        if "rel_tol" in k:
            assert abs(v - k["value"]) <= k["rel_tol"] * abs(k["value"]), (k, v)
        else:
            assert abs(v - k["value"]) <= k["abs_tol"], (k, v)


def test_tables_basic_properties(oracle_mod, he4gpu_mod):
    cfg = small_cfg(32, 32, 32, xmax=12.8)
    t = oracle_mod.build_tables(cfg)
    assert t["wcgk"][0] == 1.0  # initcg.f90:44-46
    assert t["kalfs"][0] == 1.0
    assert abs(t["fvlj4"][0] - oracle_mod.load().orc_bforce(10.22, 2.556, 2.190323)) < 1e-12
    # potion: umax inside the cutoff, V_Xe_He outside
    assert t["potion"][0] == 2793.9365463
    assert np.all(np.isfinite(t["fvlj4"]))


def test_timec_rounded_to_single(oracle_mod, he4gpu_mod):
    """timec's real part goes through a default-kind CMPLX (DFT4He3d.f90:694)."""
    cfg = small_cfg(32, 32, 32, xmax=28.0, tzmean=20.0)
    o = oracle_mod.OracleRun(cfg, oracle_mod.build_tables(cfg))
    h = 2 * 28.0 / 32
    for iz in (0, 3, 16, 31):
        z = -28.0 + h * iz
        s = 1.0 + np.tanh((abs(-28.0) - 1000.0) / 2.0)
        s = s + 1.0
        s = s + np.tanh((abs(-28.0) - 1000.0) / 2.0)
        s = s + 1.0
        s = s + np.tanh((abs(z) - 20.0) / 2.0)
        assert o.timec(0, 0, iz) == float(np.float32(2.0 * s))


def _run_pair(oracle_mod, case, nsteps, **over):
    import he4gpu
    psi, r, v, meta = he4gpu.collision_case(case)
    kw, tk = he4gpu.config_for_case(meta)
    kw.update(over)
    cfg = he4gpu.default_config(meta["nx"], meta["ny"], meta["nz"], meta["xmax"], meta["ymax"], meta["zmax"],
                                **kw)
    tabs = oracle_mod.build_tables(cfg, tk["selec"], tk["r_cutoff"], tk["umax"])
    o = oracle_mod.OracleRun(cfg, tabs)
    o.set_state(psi, r, v)
    return o, cfg, meta


def test_norm_conserved_without_absorber(oracle_mod, he4gpu_mod):
    """Real-time evolution conserves sum(den) when the absorber is off."""
    o, cfg, meta = _run_pair(oracle_mod, "he100_xe_32", 0, lambdah=0.0)
    n0 = o.den.sum()
    o.step(8)
    n1 = o.den.sum()
    assert abs(n1 - n0) / n0 < 1e-9


def test_energy_conserved_without_absorber(oracle_mod, he4gpu_mod):
    """E_tot drifts only at the level of the mismatch between the kinetic energy
    (first-derivative stencil squared, energy.f90:51-53) and the Hamiltonian's
    second-derivative stencil on this coarse (h = 0.8 A) grid."""
    o, cfg, meta = _run_pair(oracle_mod, "he100_xe_32", 0, lambdah=0.0)
    e0 = o.energy()["etot"]
    o.step(8)
    e1 = o.energy()["etot"]
    assert abs(e1 - e0) / abs(e0) < 5e-4


def test_rk_then_pc_history(oracle_mod, he4gpu_mod):
    """Three RK-Gill steps fill the history, then the PC error estimate is small."""
    o, cfg, meta = _run_pair(oracle_mod, "he100_xe_32", 0)
    o.step(3)
    eh, ei = o.step(1)
    assert 0 < eh < 1e-8
    assert ei >= 0


def test_results_do_not_depend_on_the_thread_count(oracle_mod, he4gpu_mod):
    """The oracle's sums are compensated per z plane and combined in plane
    order, so a run on one thread and on several gives the same bits: psi,
    the density, every energy component and the impurity after RK and PC
    steps (the CPU baseline may use any core count)."""
    import he4gpu
    psi, r, v, meta = he4gpu.collision_case("he100_xe_32")
    kw, tk = he4gpu.config_for_case(meta)
    cfg = he4gpu.default_config(meta["nx"], meta["ny"], meta["nz"], meta["xmax"], **kw)
    tabs = oracle_mod.build_tables(cfg, tk["selec"], tk["r_cutoff"], tk["umax"])
    lib = oracle_mod.load()
    out = []
    try:
        for threads in (1, max(2, os.cpu_count() or 2)):
            lib.orc_set_threads(threads)
            o = oracle_mod.OracleRun(cfg, tabs)
            o.set_state(psi, r, v)
            o.step(5)
            out.append((o.psi, o.den, o.energy(), o.impurity()))
            o.close()
    finally:
        lib.orc_set_threads(os.cpu_count() or 1)
    (pa, da, ea, ia), (pb, db, eb, ib) = out
    assert np.array_equal(pa, pb) and np.array_equal(da, db)
    assert ea == eb
    assert all(np.array_equal(x, y) for x, y in zip(ia, ib))
