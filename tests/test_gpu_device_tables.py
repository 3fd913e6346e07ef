"""k-space set-up tables built on the device (he4g_create with NULL fvlj4,
wcgk and kalfs: fforma.f90:36-60, initcg.f90:32-49, DFT4He3d.f90:592-596)
against the host-built tables of he4g_build_tables, through the C ABI.

The tables enter the fields linearly (dencg = w*den, delj4 = V_LJ*den), so
runs on either set of tables agree to the tables' own rounding: fields after
one evaluation to 1e-13 of their maximum, psi and the impurity after steps to
1e-12, in each arithmetic form. A device-table run also meets the oracle at
the FP64 form's step tolerance (1e-10).
"""
import numpy as np
import pytest

from helpers import make_case, oracle_run, rel_field, rel_vec

pytestmark = pytest.mark.gpu

FIELD_TOL = 1e-13
STEP_TOL = 1e-12


def pair_of_runs(cfg, tk, psi, r, v):
    import he4gpu
    runs = []
    for dev in (False, True):
        run = he4gpu.Run(cfg, selec=tk["selec"], r_cutoff=tk["r_cutoff"], umax=tk["umax"], device_tables=dev)
        run.set_state(psi, r, v)
        runs.append(run)
    return runs


@pytest.mark.parametrize("case,over", [("he100_xe_32", {}), ("he200_xe_40x48x64", {}),
                                       ("he300_ar_48", {}),
                                       ("he100_xe_32", {"core": 1, "lsolid": 0, "hcg": 2.190323})])
def test_device_tables_match_host_tables_fp64(case, over):
    cfg, tk, psi, r, v, meta = make_case(case, **over)
    host, dev = pair_of_runs(cfg, tk, psi, r, v)
    for name in ("dencg", "delj4", "pot4"):
        assert rel_field(dev.field(name), host.field(name)) < FIELD_TOL, name
    eh, ed = host.energy(), dev.energy()
    for k in eh:
        assert abs(ed[k] - eh[k]) <= 1e-12 * max(abs(eh[k]), 1e-6), k
    host.step(6)
    dev.step(6)
    assert rel_field(dev.psi, host.psi) < STEP_TOL
    assert rel_vec(dev.impurity()[0], host.impurity()[0]) < STEP_TOL
    host.close()
    dev.close()


@pytest.mark.parametrize("prec,tol", [(1, 1e-6), (2, STEP_TOL)])
def test_device_tables_in_the_mixed_and_df64_forms(prec, tol):
    """The device builder writes the run's own table type (FP32 for the mixed
    form, df64 pairs for the df64 form), rounded from the same FP64 values as
    the host upload."""
    cfg, tk, psi, r, v, meta = make_case("he100_xe_32", precision=prec)
    host, dev = pair_of_runs(cfg, tk, psi, r, v)
    host.step(5)
    dev.step(5)
    assert rel_field(dev.psi, host.psi) < tol
    host.close()
    dev.close()


def test_device_table_run_meets_the_oracle():
    import he4gpu
    cfg, tk, psi, r, v, meta = make_case("he200_xe_40x48x64")
    g = he4gpu.Run(cfg, selec=tk["selec"], r_cutoff=tk["r_cutoff"], umax=tk["umax"], device_tables=True)
    g.set_state(psi, r, v)
    o = oracle_run(cfg, tk, psi, r, v)
    g.step(7)
    o.step(7)
    assert rel_field(g.den, o.den) < 1e-10
    assert rel_vec(g.impurity()[0], o.impurity()[0]) < 1e-10
    g.close()
    o.close()


def test_one_table_pointer_alone_is_refused():
    """fvlj4 and wcgk come both from the host or both from the device."""
    import ctypes as C

    import he4gpu
    cfg, tk, psi, r, v, meta = make_case("he100_xe_32")
    t = he4gpu.build_tables(cfg, tk["selec"], tk["r_cutoff"], tk["umax"])
    lib = he4gpu.abi.load()
    h = C.c_void_p()
    rc = lib.he4g_create(C.byref(cfg), he4gpu.abi.dptr(t["fvlj4"]), None, None, he4gpu.abi.dptr(t["potion"]),
                         C.byref(h))
    assert rc == he4gpu.abi.HE4G_EINVAL
