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


def config_for_case(meta):
    """Keyword overrides of he4g_default_config for a case."""
    selec, r_cutoff, umax, mass = IMPURITIES[meta["imp"]]
    return dict(deltat=meta["dt_ps"] / KELVIN_PER_PS, mimpur=mass), dict(selec=selec, r_cutoff=r_cutoff,
                                                                         umax=umax)
