"""The oracle against a second, independent restatement in numpy of the same
Fortran lines: the mean field (poten.f90:5-118 and, for core OTC,
term_alfa.f90:5-117), one whole Runge-Kutta-Gill step (steprk.f90:21-150,
with updatepoten, poten and forceimp between its stages), and the driver loop
(DFT4He3d.f90:834-852) over three RK-Gill and three Hamming PMC steps
(steppc.f90:1-178) with their history arrays and index rotations, the
energy components (energy.f90:12-144) and the printed observables
(DFT4He3d.f90:869-943, r_cm.f90:23-58). The numpy side uses
numpy's FFTs, the 13-point rows of blockds.f (tests/golden/stencil_rows.json)
with zero padding (icon = 13), and the oracle's form-factor and impurity
tables (pinned by their own known answers). Agreement to rounding rules out a
slip in either restatement of the field formulas, the FFT scaling, the order
of the convolutions, the Gill coefficients and the impurity update."""
import json
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TOL = 1e-12  # relative to each field's maximum: FFT rounding of two implementations


def _state(nx, ny, nz, h, seed):
    rng = np.random.default_rng(seed)
    x = (np.arange(nx) - nx // 2) * h
    y = (np.arange(ny) - ny // 2) * h
    z = (np.arange(nz) - nz // 2) * h
    r = np.sqrt(z[:, None, None] ** 2 + y[None, :, None] ** 2 + x[None, None, :] ** 2)
    rho = 0.0218 / (1.0 + np.exp((r - 0.3 * nx * h) / 0.8))
    return np.sqrt(rho) * np.exp(1j * 1e-3 * rng.standard_normal(rho.shape))


def _grad1(f, axis, h, row):
    """13-point first derivative along numpy axis `axis`, zero padded."""
    n = f.shape[axis]
    pad = [(0, 0)] * 3
    pad[axis] = (6, 6)
    fp = np.pad(f, pad)
    out = np.zeros_like(f)
    for k, c in enumerate(row):
        if c == 0.0:
            continue
        sl = [slice(None)] * 3
        sl[axis] = slice(k, k + n)
        out += c * fp[tuple(sl)]
    return out / h


def _mean_field(cfg, tabs, den, row):
    shape = den.shape
    nh = (shape[0], shape[1], shape[2] // 2 + 1)
    wcgk = tabs["wcgk"].reshape(nh)
    fvlj4 = tabs["fvlj4"].reshape(nh)
    conv = lambda f, k: np.fft.irfftn(np.fft.rfftn(f) * k, s=shape, axes=(0, 1, 2))  # noqa: E731
    fden = np.fft.rfftn(den)
    dencg = np.fft.irfftn(fden * wcgk, s=shape, axes=(0, 1, 2))
    delj4 = np.fft.irfftn(fden * fvlj4, s=shape, axes=(0, 1, 2))
    g = den * dencg * (cfg.cp4 + cfg.cpp4 * dencg)
    a0, a1 = cfg.cp4 / 2.0, cfg.cpp4 / 3.0
    pot4 = delj4 + dencg ** 2 * (a0 + a1 * dencg) + conv(g, wcgk)
    out = {"dencg": dencg, "delj4": delj4}
    if cfg.core == 1:  # OTC: term_alfa
        kalfs = tabs["kalfs"].reshape(nh)
        h = [2 * cfg.xmax / cfg.nx, 2 * cfg.ymax / cfg.ny, 2 * cfg.zmax / cfg.nz]
        grads = [_grad1(den, 2 - a, h[a], row) for a in range(3)]  # x, y, z
        denalf = np.fft.irfftn(fden * kalfs, s=shape, axes=(0, 1, 2))
        falfs = 1.0 - denalf / cfg.den0s
        ints = [conv(falfs * gr, kalfs) for gr in grads]
        s1 = sum(gr * it for gr, it in zip(grads, ints))
        ua = conv(s1, kalfs) / cfg.den0s
        div = sum(_grad1(falfs * ints[a], 2 - a, h[a], row) for a in range(3))
        ualphas = (ua + div) * cfg.h2o2m4 * cfg.alphas
        pot4 = pot4 + ualphas
        out.update(denalf=denalf, ualphas=ualphas)
    if cfg.lsolid:
        t = np.tanh(cfg.beta_solid * (den - cfg.den_m))
        pot4 = pot4 + cfg.c_solid * (1.0 + t + cfg.beta_solid * den * (1.0 - t * t))
    out["pot4"] = pot4
    return out


# the odd lengths (27, 25, 45, and nx/2 = 15, 9) take the oracle's radix-3 and
# radix-5 passes on odd lines
@pytest.mark.parametrize("core,lsolid,dims", [(0, 1, (24, 20, 30)), (1, 0, (20, 24, 16)), (0, 0, (32, 32, 32)),
                                              (0, 1, (30, 27, 25)), (1, 0, (18, 45, 20))])
def test_mean_field_matches_numpy(oracle_mod, he4gpu_mod, core, lsolid, dims):
    nx, ny, nz = dims
    h = 0.45
    cfg = he4gpu_mod.default_config(nx, ny, nz, nx * h / 2, ny * h / 2, nz * h / 2, core=core, lsolid=lsolid)
    tabs = oracle_mod.build_tables(cfg)
    row = json.load(open(os.path.join(GOLDEN, "stencil_rows.json")))["d1"]["centre_row"]
    psi = _state(nx, ny, nz, h, seed=11)
    o = oracle_mod.OracleRun(cfg, tabs)
    o.set_state(psi, np.array([0.31, -0.22, -0.4 * nz * h]), np.array([0.0, 0.0, 2.0]))
    ref = _mean_field(cfg, tabs, np.abs(psi) ** 2, row)
    # The penalty's 1 + tanh(beta (rho - rho_m)) cancels to ~1e-12 inside the
    # droplet, where one ulp of tanh near -1 between two libm implementations
    # moves C (1 + t + ...) by C * 2^-53: allowed on pot4 as an absolute term.
    slack = {"pot4": 8 * 2.0 ** -53 * cfg.c_solid if lsolid else 0.0}
    for name, want in ref.items():
        got = o.field(name)
        err = np.max(np.abs(got - want))
        assert err < TOL * np.max(np.abs(want)) + slack.get(name, 0.0), (name, err)
    o.close()


def _grad2(f, axis, h, row):
    """13-point second derivative along numpy axis `axis`, zero padded."""
    return _grad1(f, axis, 1.0, row) / (h * h)


def _uimp(cfg, tabs, rimp):
    """updatepoten (potenimp.f90:71-95): int(r/d) and mod(r,d)/d."""
    h = [2 * cfg.xmax / cfg.nx, 2 * cfg.ymax / cfg.ny, 2 * cfg.zmax / cfg.nz]
    x = -cfg.xmax + h[0] * np.arange(cfg.nx)
    y = -cfg.ymax + h[1] * np.arange(cfg.ny)
    z = -cfg.zmax + h[2] * np.arange(cfg.nz)
    zt = (z - rimp[2]) ** 2
    yt = (y[None, :] - rimp[1]) ** 2 + zt[:, None]
    r = np.sqrt((x[None, None, :] - rimp[0]) ** 2 + yt[:, :, None])
    ir = (r / cfg.delinter).astype(np.int64)
    w = np.fmod(r, cfg.delinter) / cfg.delinter
    pot = tabs["potion"]
    return pot[ir] * (1.0 - w) + pot[ir + 1] * w


def _force(cfg, den, uimp, row):
    """forceimp (potenimp.f90:24-55): -sum(grad(den) * uimp) * dxyz."""
    h = [2 * cfg.xmax / cfg.nx, 2 * cfg.ymax / cfg.ny, 2 * cfg.zmax / cfg.nz]
    dxyz = h[0] * h[1] * h[2]
    return np.array([-np.sum(_grad1(den, 2 - a, h[a], row) * uimp) * dxyz for a in range(3)])


def test_rk_gill_step_matches_numpy(oracle_mod, he4gpu_mod):
    """One Runge-Kutta-Gill step (steprk.f90:21-150: four stages, the mean
    field, uimp and the force re-evaluated after stages 1-3) restated in
    numpy on the oracle's tables and timec, against the oracle's steprk."""
    gold = json.load(open(os.path.join(GOLDEN, "stencil_rows.json")))
    r1, r2 = gold["d1"]["centre_row"], gold["d2"]["centre_row"]
    nx, ny, nz, h = 24, 20, 30, 0.45
    cfg = he4gpu_mod.default_config(nx, ny, nz, nx * h / 2, ny * h / 2, nz * h / 2)
    cfg.deltat = 1.3092e-5
    tabs = oracle_mod.build_tables(cfg)
    psi = _state(nx, ny, nz, h, seed=12)
    rimp, vimp = np.array([0.31, -0.22, -5.2]), np.array([0.05, 0.0, 2.0])
    o = oracle_mod.OracleRun(cfg, tabs)
    o.set_state(psi, rimp, vimp)
    timec = o.timec_array()
    hs = [2 * cfg.xmax / nx, 2 * cfg.ymax / ny, 2 * cfg.zmax / nz]
    mass = cfg.mimpur * 0.02061484  # mimpur * mp_u (modules.f90:315, DFT4He3d.f90:205)
    # the state set_state leaves: the first evaluation, q = qr = qv = 0
    uimp = _uimp(cfg, tabs, rimp)
    den = np.abs(psi) ** 2
    pot4 = _mean_field(cfg, tabs, den, r1)["pot4"]
    aimp = _force(cfg, den, uimp, r1) / mass
    q = np.zeros_like(psi)
    qr, qv = np.zeros(3), np.zeros(3)
    s2 = np.sqrt(2.0)
    a = [0.5, 1.0 - 1.0 / s2, 1.0 + 1.0 / s2, 1.0 / 6.0]
    b = [2.0, 1.0, 1.0, 2.0]
    c = [0.5, 1.0 - 1.0 / s2, 1.0 + 1.0 / s2, 0.5]
    dt = cfg.deltat
    for j in range(4):
        lap = sum(_grad2(psi, 2 - ax, hs[ax], r2) for ax in range(3))
        s4 = timec * (lap * cfg.h2o2m4 - pot4 * psi) - 1j * uimp * psi
        s1 = a[j] * (s4 - b[j] * q)
        q = q + 3.0 * s1 - c[j] * s4
        psi = psi + dt * s1
        aux = a[j] * (vimp - b[j] * qr)
        qr = qr + 3.0 * aux - c[j] * vimp
        rimp = rimp + dt * aux
        aux = a[j] * (aimp - b[j] * qv)
        qv = qv + 3.0 * aux - c[j] * aimp
        vimp = vimp + dt * aux
        if j < 3:
            den = np.abs(psi) ** 2
            uimp = _uimp(cfg, tabs, rimp)
            pot4 = _mean_field(cfg, tabs, den, r1)["pot4"]
            aimp = _force(cfg, den, uimp, r1) / mass
    o.steprk(dt)
    assert np.max(np.abs(o.psi - psi)) < 1e-13 * np.max(np.abs(psi))
    ro, vo, ao = o.impurity()
    assert np.max(np.abs(ro - rimp)) < 1e-13 * np.max(np.abs(rimp))
    assert np.max(np.abs(vo - vimp)) < 1e-12 * np.max(np.abs(vimp))
    assert np.max(np.abs(ao - aimp)) < 1e-9 * np.max(np.abs(aimp))
    o.close()


class _NumpyRun:
    """The driver loop DFT4He3d.f90:834-852 (steprk for the first three
    steps, steppc after, then potenimp/poten/forceimp at rimp) with the
    history arrays and index rotations of steprk.f90 and steppc.f90,
    Fortran slots 1..3 as list indices 0..2."""

    def __init__(self, cfg, tabs, psi, rimp, vimp, rows):
        self.cfg, self.tabs, self.r1, self.r2 = cfg, tabs, rows[0], rows[1]
        self.h = [2 * cfg.xmax / cfg.nx, 2 * cfg.ymax / cfg.ny, 2 * cfg.zmax / cfg.nz]
        self.mass = cfg.mimpur * 0.02061484
        self.psi, self.rimp, self.vimp = psi.copy(), rimp.copy(), vimp.copy()
        self.q = np.zeros_like(psi)
        self.pc = np.zeros_like(psi)
        self.psiold = [np.zeros_like(psi) for _ in range(3)]
        self.hpsiold = [np.zeros_like(psi) for _ in range(2)]
        self.qr, self.qv, self.pcr, self.pcv = (np.zeros(3) for _ in range(4))
        self.rimpold = [np.zeros(3) for _ in range(3)]
        self.vimpold = [np.zeros(3) for _ in range(3)]
        self.aimpold = [np.zeros(3) for _ in range(2)]
        self.ioldp, self.ioldr, self.ioldv = [0, 1, 2], [0, 1, 2], [0, 1, 2]
        self.ioldh, self.iolda = [0, 1], [0, 1]
        self.timec = None
        self.nstep = 0
        self.evaluate(self.rimp)

    def evaluate(self, at):
        den = np.abs(self.psi) ** 2
        self.uimp = _uimp(self.cfg, self.tabs, at)
        self.pot4 = _mean_field(self.cfg, self.tabs, den, self.r1)["pot4"]
        self.aimp = _force(self.cfg, den, self.uimp, self.r1) / self.mass

    def hpsi(self):
        lap = sum(_grad2(self.psi, 2 - ax, self.h[ax], self.r2) for ax in range(3))
        return self.timec * (lap * self.cfg.h2o2m4 - self.pot4 * self.psi) - 1j * self.uimp * self.psi

    def steprk(self, dt):
        s2 = np.sqrt(2.0)
        a = [0.5, 1.0 - 1.0 / s2, 1.0 + 1.0 / s2, 1.0 / 6.0]
        b = [2.0, 1.0, 1.0, 2.0]
        c = [0.5, 1.0 - 1.0 / s2, 1.0 + 1.0 / s2, 0.5]
        for j in range(4):
            s4 = self.hpsi()
            s1 = a[j] * (s4 - b[j] * self.q)
            self.q = self.q + 3.0 * s1 - c[j] * s4
            if j == 0:
                self.hpsiold[1] = self.hpsiold[0]
                self.hpsiold[0] = s4
                self.psiold[2], self.psiold[1], self.psiold[0] = self.psiold[1], self.psiold[0], self.psi
            self.psi = self.psi + dt * s1
            aux = a[j] * (self.vimp - b[j] * self.qr)
            self.qr = self.qr + 3.0 * aux - c[j] * self.vimp
            if j == 0:
                self.rimpold[2], self.rimpold[1], self.rimpold[0] = self.rimpold[1], self.rimpold[0], self.rimp
            self.rimp = self.rimp + dt * aux
            aux = a[j] * (self.aimp - b[j] * self.qv)
            self.qv = self.qv + 3.0 * aux - c[j] * self.aimp
            if j == 0:
                self.aimpold[1], self.aimpold[0] = self.aimpold[0], self.aimp
                self.vimpold[2], self.vimpold[1], self.vimpold[0] = self.vimpold[1], self.vimpold[0], self.vimp
            self.vimp = self.vimp + dt * aux
            if j < 3:
                self.evaluate(self.rimp)
        self.ioldp, self.ioldr, self.ioldv = [0, 1, 2], [0, 1, 2], [0, 1, 2]
        self.ioldh, self.iolda = [0, 1], [0, 1]

    def steppc(self, dt):
        c112, c9, c4o3 = 112.0 / 121.0, 9.0 / 121.0, 4.0 / 3.0
        P, H, R, V, A = self.ioldp, self.ioldh, self.ioldr, self.ioldv, self.iolda
        s4 = self.hpsi()
        s1 = self.psiold[P[2]] + c4o3 * dt * (2.0 * s4 - self.hpsiold[H[0]] + 2.0 * self.hpsiold[H[1]])
        self.psiold[P[2]] = self.psi
        self.psi = s1 - c112 * self.pc
        self.pc = s1
        self.hpsiold[H[1]] = s4
        H[0], H[1] = H[1], H[0]
        aux = self.rimpold[R[2]] + c4o3 * dt * (2.0 * self.vimp - self.vimpold[V[0]] + 2.0 * self.vimpold[V[1]])
        self.rimpold[R[2]] = aux - c112 * self.pcr
        self.pcr = aux
        aux = self.vimpold[V[2]] + c4o3 * dt * (2.0 * self.aimp - self.aimpold[A[0]] + 2.0 * self.aimpold[A[1]])
        self.vimpold[V[2]] = aux - c112 * self.pcv
        self.pcv = aux
        self.aimpold[A[1]] = self.aimp
        A[0], A[1] = A[1], A[0]
        self.evaluate(self.rimpold[R[2]])
        s4 = self.hpsi()
        s5 = 0.125 * (9.0 * self.psiold[P[2]] - self.psiold[P[1]]
                      + 3.0 * dt * (s4 + 2.0 * self.hpsiold[H[0]] - self.hpsiold[H[1]]))
        self.pc = self.pc - s5
        self.psi = s5 + c9 * self.pc
        P[0], P[1], P[2] = P[2], P[0], P[1]
        aux = 0.125 * (9.0 * self.rimp - self.rimpold[R[1]]
                       + 3.0 * dt * (self.vimpold[V[2]] + 2.0 * self.vimp - self.vimpold[V[0]]))
        self.pcr = self.pcr - aux
        self.rimpold[R[2]] = self.rimp
        self.rimp = aux + c9 * self.pcr
        R[0], R[1], R[2] = R[2], R[0], R[1]
        aux = 0.125 * (9.0 * self.vimp - self.vimpold[V[1]]
                       + 3.0 * dt * (self.aimp + 2.0 * self.aimpold[A[0]] - self.aimpold[A[1]]))
        self.pcv = self.pcv - aux
        self.vimpold[V[2]] = self.vimp
        self.vimp = aux + c9 * self.pcv
        V[0], V[1], V[2] = V[2], V[0], V[1]

    def step(self, dt):
        self.nstep += 1
        if self.nstep <= 3:
            self.steprk(dt)
        else:
            self.steppc(dt)
        self.evaluate(self.rimp)


@pytest.mark.parametrize("dims,core", [((20, 24, 16), 0), ((18, 27, 25), 0), ((20, 24, 16), 1)])
def test_rk_and_pc_steps_match_numpy(oracle_mod, he4gpu_mod, dims, core):
    """Three Runge-Kutta-Gill steps and three Hamming predictor-modifier-
    corrector steps (steppc.f90:1-178, the impurity predictor stored into
    rimpold(:,ioldr(3)) and the field evaluated there) of the driver loop,
    restated in numpy, against the oracle's step (also on odd lengths, and
    with core OTC: lsolid off, the alpha_s term in every evaluation)."""
    gold = json.load(open(os.path.join(GOLDEN, "stencil_rows.json")))
    rows = (gold["d1"]["centre_row"], gold["d2"]["centre_row"])
    nx, ny, nz = dims
    h = 0.45
    otc = {"core": 1, "lsolid": 0, "hcg": 2.190323} if core else {}
    cfg = he4gpu_mod.default_config(nx, ny, nz, nx * h / 2, ny * h / 2, nz * h / 2, **otc)
    cfg.deltat = 1.3092e-5
    tabs = oracle_mod.build_tables(cfg)
    psi = _state(nx, ny, nz, h, seed=13)
    rimp, vimp = np.array([0.27, -0.31, -2.9]), np.array([0.04, -0.02, 2.0])
    o = oracle_mod.OracleRun(cfg, tabs)
    o.set_state(psi, rimp, vimp)
    ref = _NumpyRun(cfg, tabs, psi, rimp, vimp, rows)
    ref.timec = o.timec_array()
    for n in range(6):
        ref.step(cfg.deltat)
        o.step(1)
        assert np.max(np.abs(o.psi - ref.psi)) < 1e-12 * np.max(np.abs(ref.psi)), n
        ro, vo, ao = o.impurity()
        assert np.max(np.abs(ro - ref.rimp)) < 1e-13 * np.max(np.abs(ref.rimp)), n
        assert np.max(np.abs(vo - ref.vimp)) < 1e-11 * np.max(np.abs(ref.vimp)), n
        assert np.max(np.abs(ao - ref.aimp)) < 1e-8 * np.max(np.abs(ref.aimp)), n
    o.close()


def _energy(cfg, tabs, psi, rimp, vimp, r1):
    """energy.f90:12-144 on a state (psi, impurity at rimp with velocity vimp)."""
    h = [2 * cfg.xmax / cfg.nx, 2 * cfg.ymax / cfg.ny, 2 * cfg.zmax / cfg.nz]
    dxyz = h[0] * h[1] * h[2]
    den = np.abs(psi) ** 2
    mf = _mean_field(cfg, tabs, den, r1)
    dencg, delj4 = mf["dencg"], mf["delj4"]
    e = {}
    e["ekin4"] = cfg.h2o2m4 * sum(np.sum(np.abs(_grad1(psi, 2 - a, h[a], r1)) ** 2) for a in range(3)) * dxyz
    e["elj4"] = 0.5 * np.sum(delj4 * den) * dxyz
    e["ecor4"] = np.sum(den * dencg ** 2 * (0.5 * cfg.cp4 + cfg.cpp4 / 3.0 * dencg)) * dxyz
    e["esolid"] = 0.0
    if cfg.lsolid:
        e["esolid"] = cfg.c_solid * np.sum(den * (1.0 + np.tanh(cfg.beta_solid * (den - cfg.den_m)))) * dxyz
    e["ealphas"] = 0.0
    if cfg.core == 1:
        nh = (den.shape[0], den.shape[1], den.shape[2] // 2 + 1)
        kalfs = tabs["kalfs"].reshape(nh)
        fden = np.fft.rfftn(den)
        denalf = np.fft.irfftn(fden * kalfs, s=den.shape, axes=(0, 1, 2))
        falfs = 1.0 - denalf / cfg.den0s
        grads = [_grad1(den, 2 - a, h[a], r1) for a in range(3)]
        ints = [np.fft.irfftn(np.fft.rfftn(falfs * g) * kalfs, s=den.shape, axes=(0, 1, 2)) for g in grads]
        e["ealphas"] = -cfg.h2o2m4 * 0.5 * cfg.alphas * np.sum(falfs * sum(g * i for g, i in zip(grads, ints))) * dxyz
    e["eext"] = 0.0
    e["etot4"] = e["ekin4"] + e["elj4"] + e["ecor4"] + e["esolid"] + e["ealphas"]
    e["ekinx"] = 0.5 * cfg.mimpur * 0.02061484 * np.sum(vimp * vimp)
    e["eHeX"] = np.sum(_uimp(cfg, tabs, rimp) * den) * dxyz
    e["eimpu"] = e["ekinx"] + e["eHeX"]
    e["etot"] = e["etot4"] + e["eimpu"]
    return e, np.sum(den) * dxyz


@pytest.mark.parametrize("core,lsolid,dims", [(0, 1, (24, 20, 30)), (1, 0, (24, 20, 30)), (0, 1, (30, 27, 25))])
def test_energy_matches_numpy(oracle_mod, he4gpu_mod, core, lsolid, dims):
    """energy.f90 restated in numpy on the oracle's state, at set_state and
    after 4 steps; each component to 1e-12 of its size (the solid term, whose
    1 + tanh cancels to ~1e-12, to 8 ulps of C * N on the same libm argument)."""
    gold = json.load(open(os.path.join(GOLDEN, "stencil_rows.json")))
    r1 = gold["d1"]["centre_row"]
    nx, ny, nz = dims
    h = 0.45
    cfg = he4gpu_mod.default_config(nx, ny, nz, nx * h / 2, ny * h / 2, nz * h / 2, core=core, lsolid=lsolid)
    cfg.deltat = 1.3092e-5
    tabs = oracle_mod.build_tables(cfg)
    o = oracle_mod.OracleRun(cfg, tabs)
    o.set_state(_state(nx, ny, nz, h, seed=14), np.array([0.21, 0.33, -5.0]), np.array([0.1, 0.0, 2.0]))
    for steps in (0, 4):
        if steps:
            o.step(steps)
        r, v, _ = o.impurity()
        want, npart = _energy(cfg, tabs, o.psi, r, v, r1)
        got = o.energy()
        slack = 8 * 2.0 ** -53 * cfg.c_solid * npart if lsolid else 0.0
        for k, w in want.items():
            tol = 1e-12 * abs(w) + (slack if k in ("esolid", "etot4", "etot") else 0.0) + 1e-300
            assert abs(got[k] - w) <= tol, (steps, k, got[k], w)
    o.close()


@pytest.mark.parametrize("dims", [(24, 20, 30), (30, 27, 25)])
def test_observables_match_numpy(oracle_mod, he4gpu_mod, dims):
    """The printed observables of DFT4He3d.f90:869-943: the particle number,
    the centre of mass (r_cm.f90:23-58, divided by the namelist's n4), the
    angular momentum <L> about it from the 13-point first derivatives of psi,
    and <x^2>, <y^2>, <z^2>."""
    gold = json.load(open(os.path.join(GOLDEN, "stencil_rows.json")))
    r1 = gold["d1"]["centre_row"]
    nx, ny, nz = dims
    h = 0.45
    cfg = he4gpu_mod.default_config(nx, ny, nz, nx * h / 2, ny * h / 2, nz * h / 2)
    tabs = oracle_mod.build_tables(cfg)
    psi = _state(nx, ny, nz, h, seed=15)
    # a phase that carries angular momentum about an off-centre axis
    x = -cfg.xmax + h * np.arange(nx)
    y = -cfg.ymax + h * np.arange(ny)
    z = -cfg.zmax + h * np.arange(nz)
    psi = psi * np.exp(1j * 0.3 * (x[None, None, :] * 0.2 - y[None, :, None] * 0.5 + z[:, None, None] * 0.1))
    o = oracle_mod.OracleRun(cfg, tabs)
    o.set_state(psi, np.array([0.2, 0.1, -5.0]), np.array([0.0, 0.0, 2.0]))
    n4 = 300.0
    got = o.observables(n4)
    den = np.abs(psi) ** 2
    dxyz = h ** 3
    cm = [np.sum(den * x[None, None, :]) * dxyz / n4, np.sum(den * y[None, :, None]) * dxyz / n4,
          np.sum(den * z[:, None, None]) * dxyz / n4]
    d = [_grad1(psi, 2 - a, h, r1) for a in range(3)]  # d/dx, d/dy, d/dz
    X, Y, Z = x[None, None, :] - cm[0], y[None, :, None] - cm[1], z[:, None, None] - cm[2]
    cps = np.conj(psi)
    lz = np.sum(1j * cps * (Y * d[0] - X * d[1])) * dxyz
    ly = np.sum(1j * cps * (X * d[2] - Z * d[0])) * dxyz
    lx = np.sum(1j * cps * (Z * d[1] - Y * d[2])) * dxyz
    r2 = [np.sum(den * x[None, None, :] ** 2) * dxyz, np.sum(den * y[None, :, None] ** 2) * dxyz,
          np.sum(den * z[:, None, None] ** 2) * dxyz]
    assert abs(got["npart"] - np.sum(den) * dxyz) < 1e-13 * np.sum(den) * dxyz
    np.testing.assert_allclose(got["cm"], cm, rtol=1e-12, atol=1e-14)
    lref = np.array([lx, ly, lz])
    scale = np.max(np.abs(lref))
    assert np.max(np.abs(np.array(got["ang"]) - lref.real)) < 1e-11 * scale
    assert np.max(np.abs(np.array(got["ang_im"]) - lref.imag)) < 1e-11 * scale
    np.testing.assert_allclose(got["r2"], r2, rtol=1e-12)
    o.close()
