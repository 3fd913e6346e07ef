"""Grid lengths: every length the library accepts (2^a 3^b 5^c from 16 to
320, he4g_create) sits on an axis of the grids below: every even length as
nx (so every half-length nx/2 of the x passes' packed complex lines, odd ones
included) and every length as ny or nz (the y lines and the z convolution
columns), with nx = 2 mod 4 among them (the mixed form's scalar force
kernel). On each grid the mean-field evaluation and five steps (three
Runge-Kutta-Gill, two predictor-corrector: steprk.f90:21-150,
steppc.f90:1-178, poten.f90:5-118) are compared with the FP64 oracle:
- FP64 with the default passes (register engine where a length has a
  specialisation, the generic mixed-radix kernels elsewhere) and with the
  generic kernels for every pass;
- df64 (its tolerances equal FP64's, uimp to 2e-12 of its maximum);
- mixed (FP32 fields: 1e-5).
Some grids also run core OTC, hx, hy and hz all different, or core OT
without the solid penalty, in all three forms. The states are a seeded
Woods-Saxon density (R = 8, a = 2 Angstrom, cut by the smaller boxes) with
random phases, and the impurity sits off the grid's axes inside the box.
"""
import numpy as np
import pytest

from helpers import oracle_run, rel_field, rel_vec

FP64, MIXED, DF64 = 0, 1, 2
FIELD_TOL = 1e-12
STEP_TOL = 1e-10
DF64_UIMP_TOL = 2e-12
MIXED_TOL = 1e-5
H = 0.4
NSTEPS = 5
# the evaluation's fields and the density gradients of forceimp (derden.f90:26-28)
FIELDS = ("dencg", "delj4", "pot4", "dxden", "dyden", "dzden")
XE = {"selec": "Xe_He", "r_cutoff": 2.55, "umax": 2793.9365463}


def smooth(n):
    for p in (2, 3, 5):
        while n % p == 0:
            n //= p
    return n == 1


LENGTHS = [n for n in range(16, 321) if smooth(n)]

# the long x lines with pairs of y/z lengths (the longest with the shortest),
# the short x lines with short or odd y/z lengths, then the long even lengths
# on y or z
GRIDS = [
    (320, 243, 16), (300, 225, 18), (288, 135, 20), (270, 128, 24), (256, 125, 25),
    (250, 120, 27), (240, 108, 30), (216, 100, 32), (200, 96, 36), (192, 90, 40),
    (180, 81, 45), (162, 80, 48), (160, 75, 50), (150, 72, 54), (144, 64, 60),
    (16, 81, 25), (18, 75, 27), (20, 45, 54), (24, 27, 75), (30, 25, 81),
    (32, 54, 45), (36, 50, 27), (40, 36, 25), (48, 30, 27), (50, 24, 45),
    (54, 20, 25), (60, 18, 27), (64, 16, 45), (72, 25, 20), (80, 27, 18),
    (90, 45, 16), (96, 25, 24), (100, 27, 20), (108, 18, 25), (120, 16, 27),
    (128, 20, 25),
    (16, 320, 18), (18, 16, 300), (20, 288, 16), (24, 18, 270), (16, 256, 20),
    (18, 20, 250), (20, 240, 18), (16, 18, 216), (18, 200, 16), (20, 16, 192),
    (16, 180, 20), (18, 20, 162), (20, 160, 18), (16, 18, 150), (18, 144, 16),
]


def test_grids_cover_every_length_in_every_role():
    """Every even length appears as nx (so every nx/2 the x passes take) and
    every length as ny or nz."""
    xs = {g[0] for g in GRIDS}
    ys = {g[1] for g in GRIDS}
    zs = {g[2] for g in GRIDS}
    for g in GRIDS:
        assert g[0] % 2 == 0 and all(n in LENGTHS for n in g), g
    assert {n for n in LENGTHS if n % 2 == 0} <= xs
    assert set(LENGTHS) <= ys | zs
    assert any(g[0] % 4 == 2 for g in GRIDS) and any(g[0] % 4 == 0 for g in GRIDS)
    assert all(n in ys | zs for n in (25, 27, 45, 75, 81, 125, 135, 225, 243))


def droplet(nx, ny, nz, seed, h=(H, H, H)):
    rng = np.random.default_rng(seed)
    ext = (0.5 * h[0] * nx, 0.5 * h[1] * ny, 0.5 * h[2] * nz)
    x = -ext[0] + h[0] * np.arange(nx)
    y = -ext[1] + h[1] * np.arange(ny)
    z = -ext[2] + h[2] * np.arange(nz)
    r = np.sqrt(z[:, None, None] ** 2 + y[None, :, None] ** 2 + x[None, None, :] ** 2)
    rho = 0.0218 / (1.0 + np.exp((r - 8.0) / 2.0))
    psi = np.sqrt(rho) * np.exp(1j * 1e-3 * rng.standard_normal(rho.shape))
    rimp = np.array([0.3 * ext[0] + 0.017, -0.2 * ext[1] - 0.013, 0.25 * ext[2] + 0.031])
    return psi, rimp, np.array([0.0, 0.0, 2.0]), ext


def config(grid, ext, precision):
    import he4gpu
    cfg = he4gpu.default_config(*grid, *ext, precision=precision)
    cfg.deltat = 1.3092e-5
    return cfg


@pytest.mark.gpu
@pytest.mark.parametrize("grid", GRIDS, ids=lambda g: "x".join(map(str, g)))
def test_grid_matches_oracle(grid):
    import he4gpu
    psi, r, v, ext = droplet(*grid, seed=sum(grid))
    o = oracle_run(config(grid, ext, FP64), XE, psi, r, v)
    ref = {name: o.field(name) for name in ("uimp",) + FIELDS}
    ref_energy = o.energy()
    o.step(NSTEPS)
    ref_den, ref_psi, ref_pot4 = o.den, o.psi, o.field("pot4")
    ref_r, ref_v, _ = o.impurity()
    o.close()
    forms = [(FP64, False), (FP64, True), (DF64, False), (MIXED, False)]
    for prec, generic in forms:
        what = f"{grid} precision {prec}{' generic' if generic else ''}"
        g = he4gpu.Run(config(grid, ext, prec), **XE)
        if generic:
            t = list(g.tiles)
            t[4] = 0
            g.tiles = tuple(t)
        g.set_state(psi, r, v)
        field_tol = MIXED_TOL if prec == MIXED else FIELD_TOL
        step_tol = MIXED_TOL if prec == MIXED else STEP_TOL
        uimp = g.field("uimp")
        if prec == FP64:
            assert np.array_equal(uimp, ref["uimp"]), what
        else:
            uimp_tol = MIXED_TOL if prec == MIXED else DF64_UIMP_TOL
            assert rel_field(uimp, ref["uimp"]) < uimp_tol, what
        for name in FIELDS:
            assert rel_field(g.field(name), ref[name]) < field_tol, (what, name)
        if prec == FP64 and not generic:
            e = g.energy()
            for k in ref_energy:
                assert abs(e[k] - ref_energy[k]) <= 1e-11 * max(abs(ref_energy[k]), 1e-6), (what, k)
        g.step(NSTEPS)
        assert rel_field(g.den, ref_den) < step_tol, what
        assert rel_field(g.psi, ref_psi) < step_tol, what
        assert rel_field(g.field("pot4"), ref_pot4) < step_tol, what
        rg, vg, _ = g.impurity()
        imp_tol = 1e-8 if prec == MIXED else STEP_TOL
        assert rel_vec(rg, ref_r) < imp_tol and rel_vec(vg, ref_v) < (1e-6 if prec == MIXED else STEP_TOL), what
        g.close()


# core OTC (lsolid off): the alpha_s term's own transforms and first-derivative
# sweeps (term_alfa.f90:5-117) on grids with odd and generic-engine lengths
OTC_GRIDS = [(270, 128, 24), (18, 75, 27), (54, 20, 25), (16, 18, 216), (150, 72, 54)]


@pytest.mark.gpu
@pytest.mark.parametrize("grid", OTC_GRIDS, ids=lambda g: "x".join(map(str, g)))
def test_otc_grid_matches_oracle(grid):
    import he4gpu
    psi, r, v, ext = droplet(*grid, seed=sum(grid) + 1)
    otc = {"core": 1, "lsolid": 0, "hcg": 2.190323}

    def cfg_of(prec):
        c = config(grid, ext, prec)
        for k, x in otc.items():
            setattr(c, k, x)
        return c

    o = oracle_run(cfg_of(FP64), XE, psi, r, v)
    names = ("denalf", "ualphas", "pot4", "dencg")
    ref = {name: o.field(name) for name in names}
    ref_ealphas = o.energy()["ealphas"]
    assert ref_ealphas != 0.0
    o.step(NSTEPS)
    ref_den = o.den
    o.close()
    for prec in (FP64, DF64, MIXED):
        g = he4gpu.Run(cfg_of(prec), **XE)
        g.set_state(psi, r, v)
        # the mixed form's alpha_s term (FP32 derivatives and products) to 1e-4
        tol = 1e-4 if prec == MIXED else FIELD_TOL
        for name in names:
            assert rel_field(g.field(name), ref[name]) < tol, (grid, prec, name)
        etol = 1e-4 if prec == MIXED else 1e-11
        assert abs(g.energy()["ealphas"] - ref_ealphas) <= etol * abs(ref_ealphas), (grid, prec)
        g.step(NSTEPS)
        assert rel_field(g.den, ref_den) < (MIXED_TOL if prec == MIXED else STEP_TOL), (grid, prec)
        g.close()


# hx, hy and hz all different (the reference takes xmax, ymax and zmax apart):
# the stencils' per-axis coefficients and the form factors of a non-cubic
# momentum grid
SPACED = [((32, 32, 32), (0.4, 0.45, 0.35)), ((40, 48, 64), (0.45, 0.35, 0.4)),
          ((54, 20, 25), (0.35, 0.4, 0.45)), ((96, 24, 18), (0.42, 0.38, 0.44))]


@pytest.mark.gpu
@pytest.mark.parametrize("grid,h", SPACED, ids=lambda x: "x".join(map(str, x)))
def test_unequal_spacing_matches_oracle(grid, h):
    import he4gpu
    psi, r, v, ext = droplet(*grid, seed=sum(grid) + 2, h=h)
    o = oracle_run(config(grid, ext, FP64), XE, psi, r, v)
    ref = {name: o.field(name) for name in ("uimp", "dencg", "delj4", "pot4")}
    o.step(NSTEPS + 1)
    ref_den, ref_psi = o.den, o.psi
    ref_r, ref_v, _ = o.impurity()
    ref_energy = o.energy()
    o.close()
    for prec in (FP64, DF64, MIXED):
        what = f"{grid} h={h} precision {prec}"
        g = he4gpu.Run(config(grid, ext, prec), **XE)
        g.set_state(psi, r, v)
        tol = MIXED_TOL if prec == MIXED else FIELD_TOL
        if prec == FP64:
            assert np.array_equal(g.field("uimp"), ref["uimp"]), what
        for name in ("dencg", "delj4", "pot4"):
            assert rel_field(g.field(name), ref[name]) < tol, (what, name)
        g.step(NSTEPS + 1)
        tol = MIXED_TOL if prec == MIXED else STEP_TOL
        assert rel_field(g.den, ref_den) < tol, what
        assert rel_field(g.psi, ref_psi) < tol, what
        rg, vg, _ = g.impurity()
        assert rel_vec(rg, ref_r) < (1e-8 if prec == MIXED else STEP_TOL), what
        assert rel_vec(vg, ref_v) < (1e-6 if prec == MIXED else STEP_TOL), what
        e = g.energy()
        for k in ("etot", "ekin4", "elj4", "ecor4", "eHeX"):
            assert abs(e[k] - ref_energy[k]) <= tol * max(abs(ref_energy[k]), 1.0), (what, k)
        g.close()


@pytest.mark.gpu
@pytest.mark.parametrize("grid", [(48, 30, 27), (250, 120, 27)], ids=lambda g: "x".join(map(str, g)))
def test_ot_without_the_solid_penalty(grid):
    """Core OT with lsolid off: pot4 without the penalty term (poten.f90:110-114)
    and the energy without E_solid."""
    import he4gpu
    psi, r, v, ext = droplet(*grid, seed=sum(grid) + 3)

    def cfg_of(prec):
        c = config(grid, ext, prec)
        c.lsolid = 0
        return c

    o = oracle_run(cfg_of(FP64), XE, psi, r, v)
    ref_pot4 = o.field("pot4")
    o.step(NSTEPS)
    ref_den = o.den
    ref_energy = o.energy()
    o.close()
    for prec in (FP64, DF64, MIXED):
        g = he4gpu.Run(cfg_of(prec), **XE)
        g.set_state(psi, r, v)
        tol = MIXED_TOL if prec == MIXED else FIELD_TOL
        assert rel_field(g.field("pot4"), ref_pot4) < tol, (grid, prec)
        g.step(NSTEPS)
        tol = MIXED_TOL if prec == MIXED else STEP_TOL
        assert rel_field(g.den, ref_den) < tol, (grid, prec)
        e = g.energy()
        for k in ref_energy:
            assert abs(e[k] - ref_energy[k]) <= tol * max(abs(ref_energy[k]), 1.0), (grid, prec, k)
        g.close()
