"""CPU checks of the host-side pieces of the Fortran drop-in:

- he4g_build_uext, the TiO2 surface potential of DFT4He3d.f90:760-784
  (morse.f90), against the oracle's own restatement bit for bit, and against
  known answers of the reference's constants: the 1D well depth at Re is
  -De * 1.4387752 K (an FP32 literal in morse.f90:16), the corrugated form's
  depth above x = y = 0 is the sum of its De table, and the driver's 3000 K
  cap (DFT4He3d.f90:766,775);
- he4g_read_namelist_int on a namelist echo in the layout the driver writes
  (DFT4He3d.f90:195-196): the loop cadence the Fortran wrappers read.
"""
import math

import numpy as np
import pytest


def _cfg(he4gpu_mod, n=24, xmax=12.0):
    return he4gpu_mod.default_config(n, n + 4, n + 8, xmax, xmax * 1.1, xmax * 1.2)


@pytest.mark.parametrize("lsurf3d", [False, True])
def test_uext_matches_the_oracle(he4gpu_mod, oracle_mod, lsurf3d):
    cfg = _cfg(he4gpu_mod)
    got = he4gpu_mod.build_uext(cfg, lsurf3d=lsurf3d, zsurf=-8.0)
    ref = oracle_mod.build_uext(cfg, lsurf3d=lsurf3d, zsurf=-8.0)
    assert got.shape == (cfg.nz, cfg.ny, cfg.nx)
    assert np.array_equal(got, ref)
    assert got.max() == 3000.0  # points close to the surface hit the driver's cap
    assert got.min() < 0.0  # the well


def test_surface_known_answers(oracle_mod):
    lib = oracle_mod.load()
    de_k = 39.95 * float(np.float32(1.4387752))
    assert lib.orc_morse_1d(4.3619) == pytest.approx(-de_k, rel=1e-15)
    de = [54.671500, -2.228480, 0.585194, 13.211000, 4.842040, 0.363525, 4.614530, -1.182030, 3.747220, 3.222690,
          0.333350, 0.587320]
    ze = [4.073990, 0.057537, -0.001500, -0.568990, -0.115578, -0.018127, -0.090046, 0.008590, -0.075153,
          -0.051210, -0.023349, -0.017931]
    # at x = y = 0 every cosine is 1: the well sits at z = sum(Ze) with depth sum(De)
    assert lib.orc_morse_3d(0.0, 0.0, math.fsum(ze)) == pytest.approx(-math.fsum(de), rel=1e-12)
    # one period of the corrugation later the potential repeats
    a, b = 2.9850, 6.49548
    assert lib.orc_morse_3d(a, b, 4.5) == pytest.approx(lib.orc_morse_3d(0.0, 0.0, 4.5), rel=1e-12)


NAMELIST_ECHO = """&INPUT
 TITLE='Xe + He1000, 200 m/s', FFTWPLAN=64, NTHREAD=16, NSFILES=1,
 FILEOUT='DFT4He3d.res', FILEDENIN='He1000.den', FILEDENOUT='he1000.den',
 N4=1000, MODE=2, NX=128, NY=128, NZ=128, XMAX=  28.80000000000000     ,
 NITER=       20000, PRINTPOT=F, PENER=         200, LSOLID=T,
 ITER0=           0, TIME0=  0.000000000000000E+000,
 PCURR=        1000, ICURR=           0, LAMBDAH=   2.00000000000000     ,
 SELEC='Xe_He', R_CUTOFF=   2.55000000000000     , UMAX=   2793.93654630000
 /
"""


def test_read_namelist_int(he4gpu_mod, tmp_path):
    p = tmp_path / "DFT4He3d.namelist.read"
    p.write_text(NAMELIST_ECHO)
    got = {k: he4gpu_mod.read_namelist_int(p, k) for k in ("iter0", "niter", "pener", "pcurr", "nx", "n4")}
    assert got == {"iter0": 0, "niter": 20000, "pener": 200, "pcurr": 1000, "nx": 128, "n4": 1000}
    assert he4gpu_mod.read_namelist_int(p, "PENER") == 200  # names are case-insensitive
    assert he4gpu_mod.read_namelist_int(p, "nothere") is None
    assert he4gpu_mod.read_namelist_int(tmp_path / "missing", "pener") is None
    # a name inside a quoted string is not an assignment
    q = tmp_path / "quoted.nml"
    q.write_text("&INPUT TITLE='pener=7', PENER=9 /\n")
    assert he4gpu_mod.read_namelist_int(q, "pener") == 9


def test_timec_builder_matches_the_oracle(he4gpu_mod, oracle_mod):
    """he4g_build_timec (the absorber he4g_create uploads and the host driver
    writes to timec.dat) equals the oracle's single-precision real part."""
    cfg = he4gpu_mod.default_config(24, 28, 32, 12.0, 13.0, 14.0, lambdah=2.0, txmean=9.0, txsurf=1.5,
                                    tymean=10.0, tysurf=2.0, tzmean=11.0, tzsurf=2.5)
    got = he4gpu_mod.build_timec(cfg)
    o = oracle_mod.OracleRun(cfg, oracle_mod.build_tables(cfg))
    want = o.timec_array()
    assert np.array_equal(got.astype(np.float64), want.real)
    assert np.all(want.imag == 1.0)
    o.close()
