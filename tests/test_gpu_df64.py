"""GPU parity of the df64 form (HE4G_PREC_DF64): every per-point array and
every step kernel (stencils, H.psi, the Runge–Kutta–Gill and predictor–
corrector updates, the 3D FFT convolutions, the impurity potential and the
force) in paired-FP32 arithmetic with 48-bit significands, against the FP64
CPU oracle.

Tolerances are those of the FP64 form: fields after one potential evaluation
agree to 1e-12 of their maximum; after N steps the density, psi, every energy
component, the norm and the impurity trajectory agree to 1e-10 relative.
uimp, which the FP64 form matches bit for bit, agrees to 2e-12 of its
maximum: the table coordinate t = r/delinter reaches 1e4, and its 48-bit
rounding moves the interpolation weight by about 1e-10 next to the steepest
table step.
"""
import numpy as np
import pytest

from helpers import gpu_run, make_case, oracle_run, rel, rel_field, rel_vec

pytestmark = pytest.mark.gpu

DF64 = 2
FIELD_TOL = 1e-12
UIMP_TOL = 2e-12
STEP_TOL = 1e-10


@pytest.mark.parametrize("case", ["he100_xe_32", "he300_ar_48", "he200_xe_40x48x64"])
def test_initial_evaluation(case):
    cfg, tk, psi, r, v, meta = make_case(case, precision=DF64)
    g = gpu_run(cfg, tk, psi, r, v)
    o = oracle_run(cfg, tk, psi, r, v)
    assert rel_field(g.field("uimp"), o.field("uimp")) < UIMP_TOL
    for name in ("dencg", "delj4", "pot4"):
        assert rel_field(g.field(name), o.field(name)) < FIELD_TOL, name
    for name in ("dxden", "dyden", "dzden"):
        assert rel_field(g.field(name), o.field(name)) < FIELD_TOL, name
    eg, eo = g.energy(), o.energy()
    for k in eo:
        assert abs(eg[k] - eo[k]) <= 1e-11 * max(abs(eo[k]), 1e-6), k
    g.close()
    o.close()


def test_unequal_spacings_take_the_per_axis_stencil():
    """A grid with hx, hy, hz all different (the y and z half-extents
    stretched) runs the per-axis stencil sums, where equal spacings run the
    six-neighbour sums of a cubic grid; both meet the oracle."""
    ext = (12.8, 0.9 * 12.8, 1.1 * 12.8)
    cfg, tk, psi, r, v, meta = make_case("he100_xe_32", extents=ext, precision=DF64)
    c64, *_ = make_case("he100_xe_32", extents=ext)
    assert meta["xmax"] == 12.8
    assert len({2 * cfg.xmax / cfg.nx, 2 * cfg.ymax / cfg.ny, 2 * cfg.zmax / cfg.nz}) == 3
    g = gpu_run(cfg, tk, psi, r, v)
    o = oracle_run(c64, tk, psi, r, v)
    g.step(8)
    o.step(8)
    assert rel_field(g.den, o.den) < STEP_TOL
    assert rel_field(g.psi, o.psi) < STEP_TOL
    eg, eo = g.energy(), o.energy()
    for k in eo:
        assert abs(eg[k] - eo[k]) <= STEP_TOL * max(abs(eo[k]), 1e-3), k
    g.close()
    o.close()


@pytest.mark.parametrize("case,nsteps", [("he100_xe_32", 12), ("he300_ar_48", 8), ("he200_xe_40x48x64", 7),
                                         ("he1000_xe_128", 5)])
def test_steps_match_oracle(case, nsteps):
    """3 RK-Gill + PC steps with the trailing re-evaluation (DFT4He3d.f90:840-852)."""
    cfg, tk, psi, r, v, meta = make_case(case, precision=DF64)
    g = gpu_run(cfg, tk, psi, r, v)
    o = oracle_run(cfg, tk, psi, r, v)
    eg = g.step(nsteps)
    eo = o.step(nsteps)
    assert rel_field(g.den, o.den) < STEP_TOL
    assert rel_field(g.psi, o.psi) < STEP_TOL
    assert abs(eg[0] - eo[0]) <= 1e-10 * np.max(np.abs(psi))
    rg, vg, ag = g.impurity()
    ro, vo, ao = o.impurity()
    assert rel_vec(rg, ro) < STEP_TOL and rel_vec(vg, vo) < STEP_TOL and rel_vec(ag, ao) < 1e-8
    enG, enO = g.energy(), o.energy()
    for k in enO:
        assert abs(enG[k] - enO[k]) <= STEP_TOL * max(abs(enO[k]), 1e-3), k
    assert rel(g.den.sum(), o.den.sum()) < 1e-12
    g.close()
    o.close()


def test_reference_routines_compose_like_the_driver():
    """steprk/steppc/potenimp/poten/forceimp called one by one, as the Fortran
    driver calls them, give the same state as he4g_step in the df64 form."""
    cfg, tk, psi, r, v, meta = make_case("he100_xe_32", precision=DF64)
    a = gpu_run(cfg, tk, psi, r, v)
    b = gpu_run(cfg, tk, psi, r, v)
    a.step(5)
    dt = cfg.deltat
    m = cfg.mimpur * 0.02061484
    for it in range(1, 6):
        if it <= 3:
            b.steprk(dt)
        else:
            b.steppc(dt)
        rb, vb, _ = b.impurity()
        b.potenimp(rb)
        b.poten()
        F = b.forceimp(rb)
        b.set_impurity(rb, vb, F / m)
    assert np.array_equal(b.psi, a.psi)
    assert all(np.array_equal(x, y) for x, y in zip(a.impurity(), b.impurity()))
    a.close()
    b.close()


def test_otc_alpha_s_matches_oracle():
    """Core OTC (lsolid off) in df64: term_alfa and E_alpha (term_alfa.f90,
    energy.f90:99-105) at the FP64 form's tolerances."""
    cfg, tk, psi, r, v, meta = make_case("he100_xe_32", core=1, lsolid=0, hcg=2.190323, precision=DF64)
    g = gpu_run(cfg, tk, psi, r, v)
    o = oracle_run(cfg, tk, psi, r, v)
    for name in ("denalf", "ualphas", "pot4", "dencg"):
        assert rel_field(g.field(name), o.field(name)) < FIELD_TOL, name
    for name in ("dxden", "dyden", "dzden"):
        assert rel_field(g.field(name), o.field(name)) < FIELD_TOL, name
    eg, eo = g.energy(), o.energy()
    assert eo["ealphas"] != 0.0
    assert abs(eg["ealphas"] - eo["ealphas"]) <= 1e-11 * abs(eo["ealphas"])
    g.step(5)
    o.step(5)
    assert rel_field(g.den, o.den) < STEP_TOL
    assert rel_field(g.psi, o.psi) < STEP_TOL
    eg, eo = g.energy(), o.energy()
    for k in eo:
        assert abs(eg[k] - eo[k]) <= STEP_TOL * max(abs(eo[k]), 1e-3), k
    g.close()
    o.close()


def test_df64_tracks_the_fp64_form():
    """The df64 and FP64 forms on the GPU stay within rounding of each other."""
    cfg, tk, psi, r, v, meta = make_case("he100_xe_32", precision=DF64)
    cfg64, *_ = make_case("he100_xe_32")
    a = gpu_run(cfg, tk, psi, r, v)
    b = gpu_run(cfg64, tk, psi, r, v)
    a.step(20)
    b.step(20)
    assert rel_field(a.psi, b.psi) < 1e-11
    assert rel_vec(a.impurity()[0], b.impurity()[0]) < 1e-12
    a.close()
    b.close()


def test_lengths_without_a_register_pass_run_the_generic_kernels():
    """nx/2 = 36 and nz = 72 have no register specialisation: those passes
    run the generic Stockham kernels in df64 (ny = 64 keeps the register y
    pass), and the run meets the oracle at the form's tolerances."""
    import he4gpu
    from oracle import oracle
    cfg = he4gpu.default_config(72, 64, 72, 14.4, 12.8, 14.4, precision=DF64)
    c64 = he4gpu.default_config(72, 64, 72, 14.4, 12.8, 14.4)
    for c in (cfg, c64):
        c.deltat = 1.3092e-5
    rng = np.random.default_rng(5)
    x = -14.4 + 0.4 * np.arange(72)
    y = -12.8 + 0.4 * np.arange(64)
    z = -14.4 + 0.4 * np.arange(72)
    r2 = z[:, None, None] ** 2 + y[None, :, None] ** 2 + x[None, None, :] ** 2
    rho = 0.0218 / (1.0 + np.exp((np.sqrt(r2) - 8.0) / 0.8))
    psi = np.sqrt(rho) * np.exp(1j * 1e-3 * rng.standard_normal(rho.shape))
    # off the grid's axes: a distance that is an exact multiple of the table
    # spacing is where the reference's int(r/d), mod(r,d)/d pair steps a node
    # and the one-quotient lookup of this form does not
    r, v = np.array([0.317, -0.243, -11.05]), np.array([0.0, 0.0, 2.0])
    tk = {"selec": "Xe_He", "r_cutoff": 2.55, "umax": 2793.9365463}
    g = gpu_run(cfg, tk, psi, r, v)
    assert g.tiles[4] & 1 == 0 and g.tiles[4] & 8 == 0  # x and z passes: generic kernels
    assert g.tiles[4] & 4  # y: register engine
    o = oracle_run(c64, tk, psi, r, v)
    assert rel_field(g.field("uimp"), o.field("uimp")) < UIMP_TOL
    for name in ("dencg", "delj4", "pot4"):
        assert rel_field(g.field(name), o.field(name)) < FIELD_TOL, name
    g.step(6)
    o.step(6)
    assert rel_field(g.den, o.den) < STEP_TOL
    assert rel_field(g.psi, o.psi) < STEP_TOL
    eg, eo = g.energy(), o.energy()
    for k in eo:
        assert abs(eg[k] - eo[k]) <= STEP_TOL * max(abs(eo[k]), 1e-3), k
    rg, vg, _ = g.impurity()
    ro, vo, _ = o.impurity()
    assert rel_vec(rg, ro) < STEP_TOL and rel_vec(vg, vo) < STEP_TOL
    g.close()
    o.close()


def test_generic_and_register_passes_agree():
    """Every pass on the generic kernels (tiles bits 0) against every pass on
    the register engine (the default) on the same df64 run: the same
    butterflies in another order, so equal to rounding."""
    cfg, tk, psi, r, v, meta = make_case("he300_ar_48", precision=DF64)
    a = gpu_run(cfg, tk, psi, r, v)
    b = gpu_run(cfg, tk, psi, r, v)
    assert a.tiles[4] & 15 == 15
    b.tiles = b.tiles[:4] + (0,)
    a.step(6)
    b.step(6)
    assert rel_field(b.psi, a.psi) < 1e-12
    assert rel_field(b.field("pot4"), a.field("pot4")) < 1e-12
    assert rel_vec(b.impurity()[0], a.impurity()[0]) < 1e-13
    a.close()
    b.close()


def test_split_and_fused_z_convolutions_agree():
    """The z convolution as one fused kernel or as a forward pass plus one
    product-and-inverse pass per output (tiles bit 32): the same products,
    the inverse factored in the other order, so equal to rounding."""
    cfg, tk, psi, r, v, meta = make_case("he200_xe_40x48x64", precision=DF64)
    runs = []
    for split in (0, 32):
        x = gpu_run(cfg, tk, psi, r, v)
        t = list(x.tiles)
        t[4] = 15 | split
        x.tiles = tuple(t)
        x.step(8)
        runs.append(x)
    a, b = runs
    assert rel_field(a.psi, b.psi) < 1e-12
    assert rel_vec(a.impurity()[0], b.impurity()[0]) < 1e-13
    a.close()
    b.close()
