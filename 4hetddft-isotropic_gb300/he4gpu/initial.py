"""Seeded initial states of droplet–impurity collisions.

A Woods–Saxon density rho0 / (1 + exp((r - R)/a)) with R = 2.22 N^(1/3) A,
psi = sqrt(rho) exp(i phi) with phi seeded Gaussian noise, and a Xe (or Ar)
impurity placed outside the droplet and moving toward it. This is the state
the driver builds from a density file (DFT4He3d.f90:611-632 with xlamda = 0)
and the state a `readenc` mode-0 complex-psi file holds.

Units (DFT4He3d.f90:233-249, :302): deltat[K^-1] = deltat[ps] / 7.63822291,
v[A*K] = v[A/ps] * 7.63822291; 100 m/s = 1 A/ps.
"""
import numpy as np

KELVIN_PER_PS = 7.63822291
PS_TO_K = KELVIN_PER_PS

IMPURITIES = {
    # selec, r_cutoff, umax (V_impur.f90:757-784 and the shipped input), mass in u
    "Xe": ("Xe_He", 2.55, 2793.9365463, 131.29),
    "Ar": ("Ar_He", 2.0, 8080.8095081, 39.948),
}


def grid_axes(nx, ny, nz, xmax, ymax, zmax):
    hx, hy, hz = 2 * xmax / nx, 2 * ymax / ny, 2 * zmax / nz
    return (-xmax + hx * np.arange(nx), -ymax + hy * np.arange(ny), -zmax + hz * np.arange(nz))


def woods_saxon_psi(nx, ny, nz, xmax, ymax, zmax, n4, rho0=0.0218, a=0.8, phase_sigma=1e-3, seed=0):
    """psi as complex128 of shape (nz, ny, nx) (Fortran order of psi(nx,ny,nz))."""
    x, y, z = grid_axes(nx, ny, nz, xmax, ymax, zmax)
    R = 2.22 * n4 ** (1.0 / 3.0)
    r = np.sqrt(z[:, None, None] ** 2 + y[None, :, None] ** 2 + x[None, None, :] ** 2)
    rho = rho0 / (1.0 + np.exp((r - R) / a))
    rng = np.random.default_rng(seed)
    phi = rng.normal(0.0, phase_sigma, size=(nz, ny, nx))
    return np.sqrt(rho) * np.exp(1j * phi)


CASES = {
    # the 128^3 He_1000 + Xe collision: h = 0.45 A, Xe at z = -(R + 8) A (outside
    # the box, which the table reaching 4*xmax allows), +2 A/ps along z
    "he1000_xe_128": dict(n=128, h=0.45, n4=1000, imp="Xe", b_frac=0.0, gap=8.0, v=2.0, dt_ps=1e-4,
                          steps=1000),
    # the 256^3 He_5000 + Xe collision: h = 0.4 A, impact parameter 0.5 R, 3 A/ps
    "he5000_xe_256": dict(n=256, h=0.4, n4=5000, imp="Xe", b_frac=0.5, gap=8.0, v=3.0, dt_ps=1e-4,
                          steps=2000),
    # small cases for element-wise checks against the CPU oracle
    "he100_xe_32": dict(n=32, h=0.8, n4=100, imp="Xe", b_frac=0.3, gap=2.0, v=4.0, dt_ps=1e-4, steps=20),
    "he300_ar_48": dict(n=48, h=0.6, n4=300, imp="Ar", b_frac=0.5, gap=3.0, v=5.0, dt_ps=1e-4, steps=20),
    "he200_xe_40x48x64": dict(n=(40, 48, 64), h=0.55, n4=200, imp="Xe", b_frac=0.2, gap=2.0, v=3.0,
                              dt_ps=1e-4, steps=12),
}


def collision_case(name, seed=0):
    """Returns (psi, rimp, vimp_internal, meta) of a named case."""
    c = CASES[name]
    n = c["n"]
    nx, ny, nz = (n, n, n) if isinstance(n, int) else n
    h = c["h"]
    xmax, ymax, zmax = nx * h / 2, ny * h / 2, nz * h / 2
    R = 2.22 * c["n4"] ** (1.0 / 3.0)
    psi = woods_saxon_psi(nx, ny, nz, xmax, ymax, zmax, c["n4"], seed=seed)
    rimp = np.array([c["b_frac"] * R, 0.0, -(R + c["gap"])])
    vimp = np.array([0.0, 0.0, c["v"] * KELVIN_PER_PS])
    meta = dict(c, nx=nx, ny=ny, nz=nz, xmax=xmax, ymax=ymax, zmax=zmax, R=R)
    return psi, rimp, vimp, meta


def make_meta(n, h, n4, imp, b_frac, v, dt_ps=1e-4, steps=1000, gap=8.0, seed=0):
    """A collision case built from parameters instead of a name."""
    nx, ny, nz = (n, n, n) if isinstance(n, int) else n
    R = 2.22 * n4 ** (1.0 / 3.0)
    return dict(n=n, h=h, n4=n4, imp=imp, b_frac=b_frac, gap=gap, v=v, dt_ps=dt_ps, steps=steps, nx=nx, ny=ny,
                nz=nz, xmax=nx * h / 2, ymax=ny * h / 2, zmax=nz * h / 2, R=R, seed=seed)


def state_for(meta):
    """(psi, rimp, vimp_internal) of a case built by make_meta."""
    psi = woods_saxon_psi(meta["nx"], meta["ny"], meta["nz"], meta["xmax"], meta["ymax"], meta["zmax"], meta["n4"],
                          seed=meta.get("seed", 0))
    R = meta["R"]
    rimp = np.array([meta["b_frac"] * R, 0.0, -(R + meta["gap"])])
    vimp = np.array([0.0, 0.0, meta["v"] * KELVIN_PER_PS])
    return psi, rimp, vimp


def batch_cases(count=32, seed=2024, margin=4.0):
    """Uneven collision runs for the batched form: N log-uniform in
    [300, 3000], h uniform in [0.40, 0.45] A, the smallest grid of
    {96, 128, 160}^3 whose half-width n*h/2 holds the droplet radius plus
    `margin` A (160^3 when none does), Xe at 1-6 A/ps (100-600 m/s) with
    impact parameter uniform in [0, R]. A margin of 15 A would put every run
    of this range on 160^3 (96*0.45/2 = 21.6 A < R + 15 for all N >= 300), so
    the default margin is 4 A, which spreads the runs over the three grids."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        n4 = float(np.exp(rng.uniform(np.log(300.0), np.log(3000.0))))
        h = float(rng.uniform(0.40, 0.45))
        R = 2.22 * n4 ** (1.0 / 3.0)
        grid = next((g for g in (96, 128, 160) if g * h / 2 >= R + margin), 160)
        v = float(rng.uniform(1.0, 6.0))
        b = float(rng.uniform(0.0, 1.0))
        out.append(make_meta(grid, h, n4, "Xe", b, v, seed=seed * 1000 + i))
    return out


def serve_stream(count=200, seed=7, rate_per_s=2.0, steps_range=(500, 5000), step_scale=1.0):
    """Seeded Poisson stream of collision jobs for the serving loop: grids
    from {64, 96, 128, 192, 256}^3 weighted toward small ones, N in
    [100, 5000], Xe or Ar, 1-6 A/ps, steps in steps_range (times step_scale
    for bounded measurements). Returns a list of (arrival_s, meta)."""
    rng = np.random.default_rng(seed)
    grids = np.array([64, 96, 128, 192, 256])
    weights = np.array([0.35, 0.25, 0.2, 0.12, 0.08])
    t = 0.0
    jobs = []
    for i in range(count):
        t += float(rng.exponential(1.0 / rate_per_s))
        grid = int(rng.choice(grids, p=weights))
        h = float(rng.uniform(0.40, 0.45))
        # the droplet must fit the box: R <= n*h/2 - 8 A
        rmax = grid * h / 2 - 8.0
        nmax = min(5000.0, (rmax / 2.22) ** 3)
        n4 = float(rng.uniform(100.0, max(100.0, nmax)))
        imp = "Xe" if rng.uniform() < 0.5 else "Ar"
        v = float(rng.uniform(1.0, 6.0))
        b = float(rng.uniform(0.0, 1.0))
        steps = int(max(4, round(rng.integers(steps_range[0], steps_range[1] + 1) * step_scale)))
        jobs.append((t, make_meta(grid, h, n4, imp, b, v, steps=steps, gap=4.0, seed=seed * 1000 + i)))
    return jobs


def config_for_case(meta):
    """Keyword overrides of he4g_default_config for a case."""
    selec, r_cutoff, umax, mass = IMPURITIES[meta["imp"]]
    return dict(deltat=meta["dt_ps"] / KELVIN_PER_PS, mimpur=mass), dict(selec=selec, r_cutoff=r_cutoff,
                                                                         umax=umax)
