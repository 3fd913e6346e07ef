"""Impurity-He radial potentials of V_impur.f90's Select_pot beyond Xe and
Ar: the product's host tables (csrc/setup.cpp) against the oracle's
restatement, and properties that pin each form (host-side, no GPU)."""
import numpy as np
import pytest

import he4gpu
from oracle import oracle

NEW = ["Aziz_He", "LJ_OT", "LI", "NA", "K", "RB", "CS", "null"]


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
