"""Impurity-He radial potentials of V_impur.f90's Select_pot beyond Xe and
Ar: the product's host tables (csrc/setup.cpp) against the oracle's
restatement, and properties that pin each form (host-side, no GPU)."""
import numpy as np
import pytest

import he4gpu
from oracle import oracle

NEW = ["Aziz_He", "LJ_OT", "LI", "NA", "K", "RB", "CS", "null", "Ag_gs", "Ag_Pi", "Ag_Sig", "Ba_gs", "Au",
       "Na_plus_Koutselos", "K_plus_Koutselos", "Rb_plus_Koutselos", "Cs_plus_Koutselos"]


def small_cfg():
    return he4gpu.default_config(16, 16, 16, 8.0, 8.0, 8.0)


@pytest.mark.parametrize("selec", NEW + ["Xe_He", "Ar_He"])
def test_tables_match_the_oracle(selec):
    cfg = small_cfg()
    a = he4gpu.build_tables(cfg, selec, 2.0, 1.0e4)["potion"]
    b = oracle.build_tables(cfg, selec, 2.0, 1.0e4, with_kalfs=False)["potion"]
    assert np.array_equal(a, b)
    if selec == "null":
        assert not a.any()
    else:
        assert a[0] == 1.0e4  # inside r_cutoff: umax


def test_unknown_potential_is_refused():
    with pytest.raises(he4gpu.He4gError):
        he4gpu.build_tables(small_cfg(), "Kr_He", 2.0, 1.0e4)


def test_lj_ot_is_continuous_at_its_core():
    lib = oracle.load()
    rc, fc = 2.190323254008688, 1.574659520268255e2
    assert lib.orc_v_lj_ot(rc) == fc
    assert lib.orc_v_lj_ot(rc * (1 + 1e-12)) == pytest.approx(fc, rel=1e-9)


def test_aziz_well_at_rm():
    # HFD-B: the well of depth eps = 10.948 K sits at rm = 2.963 A
    lib = oracle.load()
    v = [lib.orc_v_aziz_he(r) for r in np.linspace(2.6, 3.4, 801)]
    assert min(v) == pytest.approx(-10.948, abs=0.02)
    assert np.linspace(2.6, 3.4, 801)[int(np.argmin(v))] == pytest.approx(2.963, abs=0.01)


@pytest.mark.parametrize("elem", range(5))
def test_alkali_forms(elem):
    lib = oracle.load()
    c6 = [22.5, 24.7, 38.9, 44.6, 51.2][elem]
    c8 = [1.06e3, 1.29e3, 2.66e3, 3.18e3, 4.34e3][elem]
    k = 11604.448 * 27.211608
    # far out the density overlap and the damping vanish: -(C6/d^6 + C8/d^8)
    d = 40.0 / 0.529177249
    assert lib.orc_v_alkali_he(40.0, elem) == pytest.approx(-(c6 / d**6 + c8 / d**8) * k, rel=1e-6)
    # repulsive core, shallow well of a few K between 5 and 9 A
    assert lib.orc_v_alkali_he(3.0, elem) > 0
    r = np.linspace(4.0, 10.0, 601)
    v = np.array([lib.orc_v_alkali_he(x, elem) for x in r])
    assert -5.0 < v.min() < 0.0 and 5.0 < r[v.argmin()] < 9.0


def test_au_pins():
    """V_impur.f90:2476-2497: V(Re) = -De exactly (s = 0); Select_pot's comment
    for 'Au' (:671-673) gives r_cutoff = 1 A with umax = 6.645232E+04, the
    form's own value there."""
    lib = oracle.load()
    assert lib.orc_v_au_he(4.124) == -20.301143
    assert lib.orc_v_au_he(1.0) == pytest.approx(6.645232e4, rel=1e-6)
    r = np.linspace(3.0, 8.0, 2001)
    v = np.array([lib.orc_v_au_he(x) for x in r])
    # the fitted polynomial puts the well within 0.1 % of -De and 0.05 A of Re
    assert v.min() == pytest.approx(-20.301143, rel=1e-3) and r[v.argmin()] == pytest.approx(4.124, abs=0.05)


def test_ba_pins():
    """V_impur.f90:1194-1210: the flat core (1297.1 K up to 3.7 A) meets the
    inverse-power fit there; a shallow well (a few K) near 7 A; the leading
    x^-6 and x^-8 terms far out."""
    lib = oracle.load()
    assert lib.orc_v_ba_he(3.7) == 1297.1
    assert lib.orc_v_ba_he(3.7 * (1 + 1e-12)) == pytest.approx(1297.1, rel=1e-5)
    r = np.linspace(4.0, 12.0, 1601)
    v = np.array([lib.orc_v_ba_he(x) for x in r])
    assert -5.0 < v.min() < -2.0 and 6.0 < r[v.argmin()] < 8.0
    x = 200.0  # the two leading terms; the x^-10 one is 1.5e-5 of them here
    assert lib.orc_v_ba_he(x) == pytest.approx(-450294.6878721156 / x**6 + 4.900282758445466e7 / x**8, rel=1e-4)


@pytest.mark.parametrize("state,c6", [(0, 137042.07), (1, 0.21661134e6), (2, 1.97443e-9)])
def test_ag_pins(state, c6):
    """V_impur.f90:1035-1092: A at r = 0; undamped dispersion beyond D, so far
    out the C6..C12 series alone; an attractive well between the core and
    the tail."""
    lib = oracle.load()
    A = [78741.3877, 0.7095092e6, 40005.2][state]
    assert lib.orc_v_ag_he(0.0, state) == A
    c8, c10, c12 = [(189386.217, 111358462.0, 1.17670377e10), (123454.7952, 0.307155024e6, 0.740464032e-10),
                    (3.37393e-6, 0.00788363, 7.52624e12)][state]
    r = 40.0
    assert lib.orc_v_ag_he(r, state) == pytest.approx(-(c6 / r**6 + c8 / r**8 + c10 / r**10 + c12 / r**12), rel=1e-9)
    rr = np.linspace(2.0, 14.0, 4001)
    v = np.array([lib.orc_v_ag_he(x, state) for x in rr])
    assert v.min() < 0.0 and rr[v.argmin()] < 10.0


def test_koutselos_ions_meet_the_reference_values():
    """Select_pot's comments (V_impur.f90:240-243, 277-280) give the values at
    the cores the reference ran with: Na+ umax = 9.012825d4 at r_cutoff = 1 A;
    K+ 1.8628633412d5 at 1 A and 3.2762532479d3 at 2 A."""
    lib = oracle.load()
    assert lib.orc_v_koutselos(1.0, 0) == pytest.approx(9.012825e4, rel=1e-7)
    assert lib.orc_v_koutselos(1.0, 1) == pytest.approx(1.8628633412e5, rel=1e-10)
    assert lib.orc_v_koutselos(2.0, 1) == pytest.approx(3.2762532479e3, rel=1e-10)


@pytest.mark.parametrize("ion", range(4))
def test_koutselos_wells(ion):
    """Ion-He wells of a few hundred K between 2 and 4 A (the polarisation
    attraction of a bare ion), deepest for the smallest ion."""
    lib = oracle.load()
    r = np.linspace(1.5, 8.0, 2601)
    v = np.array([lib.orc_v_koutselos(x, ion) for x in r])
    assert -500.0 < v.min() < -100.0 and 2.0 < r[v.argmin()] < 4.0
