"""GPU checks of the entry points the unchanged Fortran driver needs, through
the C ABI:

- he4g_set_timec: a run created without an absorber and handed the driver's
  timec module array (DFT4He3d.f90:689-699; here the oracle's copy of it)
  steps bit for bit like a run whose config carries the same absorber, and
  both match the oracle; malformed arrays are refused;
- he4g_set_uext: the external potential enters the energy only
  (energy.f90:124): eext and etot4 match the oracle with the same uext, the
  fields do not move, and NULL removes it again.
"""
import numpy as np
import pytest

from helpers import gpu_run, make_case, oracle_run, rel_field

pytestmark = pytest.mark.gpu

# an absorber that reaches into the 32^3 box (|x|, |z| up to 12.8 A)
ABSORBER = dict(lambdah=2.0, txmean=10.0, txsurf=1.5, tymean=1000.0, tysurf=2.0, tzmean=9.0, tzsurf=2.0)


@pytest.mark.parametrize("precision", [0, 1, 2])
def test_set_timec_equals_the_config_absorber(precision):
    import he4gpu
    cfg_a, tk, psi, r, v, meta = make_case("he100_xe_32", precision=precision, **ABSORBER)
    cfg_0, *_ = make_case("he100_xe_32", precision=precision, lambdah=0.0)
    a = gpu_run(cfg_a, tk, psi, r, v)
    b = gpu_run(cfg_0, tk, psi, r, v)
    o = oracle_run(cfg_a, tk, psi, r, v)
    timec = o.timec_array()
    assert np.all(timec.imag == 1.0) and timec.real.max() > 0.5  # the absorber is on inside the box
    b.set_timec(timec)
    a.step(6)
    b.step(6)
    assert np.array_equal(a.psi, b.psi)
    assert all(np.array_equal(x, y) for x, y in zip(a.impurity(), b.impurity()))
    if precision == 0:
        o.step(6)
        assert rel_field(b.den, o.den) < 1e-10
    # the absorber takes norm out: without it the run conserves the norm better
    c = gpu_run(cfg_0, tk, psi, r, v)
    c.step(6)
    n0 = float(np.sum(np.abs(psi) ** 2))
    assert abs(float(np.sum(c.den)) - n0) < abs(float(np.sum(b.den)) - n0)
    for run in (a, b, c):
        run.close()
    o.close()
    del he4gpu


def test_set_timec_refuses_what_the_device_cannot_hold():
    import he4gpu
    cfg, tk, psi, r, v, meta = make_case("he100_xe_32")
    g = gpu_run(cfg, tk, psi, r, v)
    good = np.full(g.shape, 0.5 + 1j, dtype=np.complex128)
    g.set_timec(good)
    bad = good.copy()
    bad[3, 4, 5] = 0.5 + 0.5j  # imaginary part other than 1: not real-time evolution
    with pytest.raises(he4gpu.He4gError) as e:
        g.set_timec(bad)
    assert e.value.code == he4gpu.abi.HE4G_EINVAL and "timec(6,5,4)" in str(e.value)
    bad = good.copy()
    bad[0, 0, 1] = 0.1 + 1j  # 0.1 is not a single-precision value
    with pytest.raises(he4gpu.He4gError):
        g.set_timec(bad)
    g.close()


@pytest.mark.parametrize("lsurf3d,precision", [(False, 0), (True, 0), (False, 1), (True, 2)])
def test_uext_enters_the_energy_only(lsurf3d, precision):
    import he4gpu
    cfg, tk, psi, r, v, meta = make_case("he100_xe_32", precision=precision)
    cfg64, *_ = make_case("he100_xe_32")
    # the surface 1 A inside the box's lower z face: its well (4.4 A above
    # the surface) lies in the droplet's tail
    uext = he4gpu.build_uext(cfg, lsurf3d=lsurf3d, zsurf=-meta["zmax"] + 1.0)
    g = gpu_run(cfg, tk, psi, r, v)
    ref = gpu_run(cfg, tk, psi, r, v)
    o = oracle_run(cfg64, tk, psi, r, v)
    g.set_uext(uext)
    o.set_uext(uext)
    tol = 1e-11 if precision != 1 else 1e-5
    for steps in (0, 4):
        if steps:
            for run in (g, ref, o):
                run.step(steps)
        eg, eo = g.energy(), o.energy()
        assert eo["eext"] != 0.0
        assert abs(eg["eext"] - eo["eext"]) <= tol * abs(eo["eext"])
        assert abs(eg["etot4"] - eo["etot4"]) <= tol * abs(eo["etot4"])
        assert np.array_equal(g.den, ref.den)  # uext does not act on the dynamics
        assert ref.energy()["eext"] == 0.0
        assert abs(eg["etot4"] - (ref.energy()["etot4"] + eg["eext"])) <= 1e-12 * abs(eg["etot4"])
    g.set_uext(None)
    assert g.energy()["eext"] == 0.0
    for run in (g, ref, o):
        run.close()


def test_the_fortran_wrapper_call_sequence():
    """The calls the Fortran wrappers make (he4g_wrappers.f90), in the
    driver's order (DFT4He3d.f90:641-645 before the loop, :840-852 in it):
    a run created without an absorber, potenimp/poten/forceimp/energy before
    the loop, the driver's timec and uext sent at the first step, then per
    step set_impurity, steprk or steppc, get_impurity, potenimp, poten,
    forceimp and aimp = F/m on the host. It ends bit for bit where he4g_step
    on a run configured with the same absorber ends."""
    cfg_a, tk, psi, r, v, meta = make_case("he100_xe_32", **ABSORBER)
    cfg_0, *_ = make_case("he100_xe_32", lambdah=0.0)
    a = gpu_run(cfg_a, tk, psi, r, v)
    o = oracle_run(cfg_a, tk, psi, r, v)
    timec = o.timec_array()
    o.close()
    b = gpu_run(cfg_0, tk, psi, r, v)
    m = cfg_a.mimpur * 0.02061484
    rr, vv, _ = b.impurity()
    b.potenimp(rr)
    b.poten()
    aa = b.forceimp(rr) / m
    b.energy()
    nsteps = 7
    a.step(nsteps)
    for k in range(1, nsteps + 1):
        if k == 1:
            b.set_timec(timec)
            b.set_uext(np.zeros(b.shape))
        b.set_impurity(rr, vv, aa)
        if k <= 3:
            b.steprk(cfg_a.deltat)
        else:
            b.steppc(cfg_a.deltat)
        rr, vv, _ = b.impurity()
        b.potenimp(rr)
        b.poten()
        aa = b.forceimp(rr) / m
    assert np.array_equal(a.psi, b.psi)
    ra, va, aa_dev = a.impurity()
    assert np.array_equal(ra, rr) and np.array_equal(va, vv)
    assert np.array_equal(aa_dev, aa)
    assert b.energy()["eext"] == 0.0
    a.close()
    b.close()
