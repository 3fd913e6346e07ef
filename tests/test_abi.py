"""CPU checks of the C ABI: libhe4g.so loads, exports every entry point that
include/he4g.h declares, and its host-side set-up code (defaults and tables)
agrees with the oracle. No call here touches a GPU."""
import os
import re
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    text = open(os.path.join(ROOT, "include", "he4g.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(he4g_[a-z_0-9]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(he4gpu_mod):
    from he4gpu import abi
    path = abi.lib_path()
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (he4g_\w+)", out))
    declared = header_functions()
    assert declared, "no declarations parsed"
    missing = [f for f in declared if f not in exported]
    assert not missing, missing
    # and the ctypes table covers them all
    assert set(declared) <= set(abi.SIGNATURES)


def test_default_config_matches_reference_defaults(he4gpu_mod):
    cfg = he4gpu_mod.default_config(192, 192, 192, 38.4)
    # modules.f90:138-148, :209-212; deriva :27-33
    assert (cfg.npd, cfg.icon, cfg.lsolid) == (13, 13, 1)
    assert cfg.cp4 == -2.41186e4 and cfg.cpp4 == 1.85850e6
    assert cfg.h2o2m4 == 6.05969638298 and cfg.alphas == 54.31 and cfg.den0s == 0.04
    assert cfg.c_solid == 3.1577504e4 and cfg.beta_solid == 40.0 and cfg.den_m == 0.37
    assert cfg.eps4 == 10.22 and cfg.sigma4 == 2.556 and cfg.h4 == 2.190323
    assert cfg.hcg == 2.190323 * 1.065
    # potenimpini.f90:13-16
    assert cfg.npot == 100 * 192 + 1
    assert cfg.delinter == 4.0 * 38.4 / (cfg.npot - 1)


def test_python_defaults_equal_the_library(he4gpu_mod):
    """abi.reference_defaults (used where libhe4g.so must not be loaded) fills
    every field exactly as he4g_default_config does."""
    from he4gpu import abi
    for dims in ((256, 256, 256, 51.2, 51.2, 51.2), (40, 48, 64, 11.0, 13.2, 17.6), (32, 32, 32, 12.8, 12.8, 12.8)):
        lib_cfg = he4gpu_mod.default_config(*dims)
        py_cfg = abi.reference_defaults(*dims)
        for k, _ in abi.Config._fields_:
            assert getattr(py_cfg, k) == getattr(lib_cfg, k), k
    a = he4gpu_mod.reference_config(128, 128, 128, 28.8, deltat=1e-5, mimpur=39.948)
    b = he4gpu_mod.default_config(128, 128, 128, 28.8, deltat=1e-5, mimpur=39.948)
    assert bytes(a) == bytes(b)


def test_build_tables_match_oracle(he4gpu_mod, oracle_mod):
    for (n, xmax, selec, rc, um) in ((32, 12.8, "Xe_He", 2.55, 2793.9365463), (48, 14.4, "Ar_He", 2.0,
                                                                                 8080.8095081)):
        cfg = he4gpu_mod.default_config(n, n, n, xmax)
        got = he4gpu_mod.build_tables(cfg, selec, rc, um, with_kalfs=True)
        ref = oracle_mod.build_tables(cfg, selec, rc, um)
        for k in ("fvlj4", "wcgk", "kalfs", "potion"):
            a, b = got[k], ref[k]
            assert np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300)) < 1e-13, k


def test_run_fails_loudly_without_library(monkeypatch, he4gpu_mod):
    """The Python host never falls back: a missing library is an error."""
    from he4gpu import abi, build
    monkeypatch.setattr(abi, "_lib", None)
    monkeypatch.setattr(build, "LIB", os.path.join(ROOT, "does", "not", "exist.so"))
    try:
        abi.load(build_if_missing=False)
    except RuntimeError as e:
        assert "missing" in str(e)
    else:
        raise AssertionError("load() did not fail")
