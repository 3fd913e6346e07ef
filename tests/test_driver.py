"""The native host driver (4hetddft-isotropic_gb300/host/he4g_driver.cpp), a
stand-in for DFT4He3d.f90 over the C ABI: its namelist reading against the
Python reader (CPU), and on the GPU its trajectory files, energy blocks and
density dump against the same run driven through the Python mirror."""
import os
import re
import subprocess

import numpy as np
import pytest

import he4gpu
from he4gpu import build, formats

# the reference's shipped input, as DFT4He3d.f90 reads it (grid and time step
# made small; the rest kept)
NAMELIST = """ &input
 Lambdah = 2.d0
 tzmean = 49.2d0
 tzsurf = 2.d0
 mimpur = 131.29d0
 nthread = 5
 lsurf = .FALSE.
 title = '4He_1000 + Xe'
 n4 = 1000
 icurr = 0
 iter0 = 0
 time0 = 0
 mode = {mode}
 selec = 'Xe_He'
 r_cutoff = 2.55d0
 umax = 2.7939365463E+03
 filedenin  = '{filein}'
 nx = {nx}
 ny = {ny}
 nz = {nz}
 xmax = {xmax}d0
 ymax = {ymax}d0
 zmax = {zmax}d0
 npd=13
 core4='OT'
 niter={niter}
 icon=13
 ximp= -27.0d0
 yimp= 0.0d0
 zimp= 0.0d0
 pener={pener}
 pcurr  = {pcurr}
 deltatps=1.d-4
 lrkpc=.true.
 vximp = 2.00d0
 vyimp = 0.00d0
 vzimp = 0.00d0
 /
"""


def driver():
    build.build()
    return build.DRIVER


@pytest.mark.parametrize("n,ext", [((192, 192, 192), (38.4, 38.4, 38.4)), ((40, 48, 64), (9.0, 9.6, 12.8))])
def test_parse_matches_the_python_reader(tmp_path, n, ext):
    text = NAMELIST.format(mode=0, filein="den.in", nx=n[0], ny=n[1], nz=n[2], xmax=ext[0], ymax=ext[1],
                           zmax=ext[2], niter=99999999, pener=200, pcurr=2000)
    nml = tmp_path / "input.nml"
    nml.write_text(text)
    out = subprocess.run([driver(), str(nml), "--parse"], capture_output=True, text=True, check=True).stdout
    got = dict(kv.split("=", 1) for kv in out.split())
    cfg, over, table, rimp, vimp, loop = formats.run_from_namelist(formats.read_namelist(str(nml)))
    assert (int(got["nx"]), int(got["ny"]), int(got["nz"])) == (cfg["nx"], cfg["ny"], cfg["nz"]) == n
    assert (float(got["xmax"]), float(got["ymax"]), float(got["zmax"])) == (cfg["xmax"], cfg["ymax"], cfg["zmax"])
    assert float(got["deltat"]) == over["deltat"]
    assert float(got["mimpur"]) == over["mimpur"] and float(got["tzmean"]) == over["tzmean"]
    assert float(got["lambdah"]) == over["lambdah"]
    assert got["selec"] == table["selec"] and float(got["umax"]) == table["umax"]
    assert [float(x) for x in got["rimp"].split(",")] == list(rimp)
    assert [float(x) for x in got["vimp"].split(",")] == list(vimp)
    assert int(got["pener"]) == loop["pener"] and int(got["pcurr"]) == loop["pcurr"]
    assert got["filedenin"] == "den.in" and int(got["lsolid"]) == 1 and int(got["core"]) == 0


def fortran_rows(path):
    rows = []
    for line in open(path):
        if line.startswith("#"):
            continue
        # (1x,1p,E15.6,3E18.10): fixed-width fields, one digit before the point
        assert len(line) == 1 + 15 + 3 * 18 + 1, line
        fields = [line[1:16]] + [line[16 + 18 * k:34 + 18 * k] for k in range(3)]
        assert re.fullmatch(r" *-?\d\.\d{6}E[+-]\d{2}", fields[0]), line
        assert all(re.fullmatch(r" *-?\d\.\d{10}E[+-]\d{2}", f) for f in fields[1:]), line
        rows.append([float(x) for x in fields])
    return np.array(rows)


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["he100_xe_32", "he200_xe_40x48x64"])
def test_driver_outputs_match_the_python_mirror(tmp_path, case):
    psi, r, v, meta = he4gpu.collision_case(case)
    nx, ny, nz = meta["nx"], meta["ny"], meta["nz"]
    xmax, ymax, zmax = meta["xmax"], meta["ymax"], meta["zmax"]
    psi_f = psi.reshape(nz, ny, nx).transpose(2, 1, 0)  # (nx, ny, nz), x fastest in memory order F
    den_in = tmp_path / "den.in"
    formats.write_density(str(den_in), psi_f, r, v, xmax, ymax, zmax)
    niter, pener, pcurr = 8, 4, 8
    (tmp_path / "input.nml").write_text(NAMELIST.format(mode=2, filein=str(den_in), nx=nx, ny=ny, nz=nz, xmax=xmax,
                                                        ymax=ymax, zmax=zmax, niter=niter, pener=pener,
                                                        pcurr=pcurr))
    res = subprocess.run([driver(), "input.nml"], capture_output=True, text=True, cwd=tmp_path)
    assert res.returncode == 0, res.stderr

    # the same run through the Python mirror (device-built tables, as the driver's)
    kw, tk = he4gpu.config_for_case(dict(meta, dt_ps=1e-4, imp="Xe"))
    cfg = he4gpu.default_config(nx, ny, nz, xmax, ymax, zmax, lambdah=2.0, tzmean=49.2, tzsurf=2.0, **kw)
    run = he4gpu.Run(cfg, selec="Xe_He", r_cutoff=2.55, umax=2793.9365463, device_tables=True)
    run.set_state(psi, r, v)
    want_r, energies = [run.impurity()[0]], {}
    for it in range(1, niter + 1):
        run.step(1)
        want_r.append(run.impurity()[0])
        if it % pener == 0:
            energies[it] = run.energy()

    rr = fortran_rows(tmp_path / "rimp.out")
    assert rr.shape == (niter + 1, 4)
    assert np.allclose(rr[:, 0], -1.0 * 0 + np.arange(niter + 1) * 1e-4)  # time0 = 0 in this input
    assert np.allclose(rr[:, 1:], np.array(want_r), rtol=1e-9, atol=1e-9)
    fortran_rows(tmp_path / "vimp.out")
    fortran_rows(tmp_path / "aimp.out")

    blocks = re.findall(r"Total Energy \(He\)\.+ +(-?\d+\.\d{6}) K", res.stdout)
    assert len(blocks) == niter // pener
    for k, it in enumerate(sorted(energies)):
        assert float(blocks[k]) == pytest.approx(energies[it]["etot4"], abs=2e-6)
    assert res.stdout.count("Error( He, imp) (From Steppc)") == niter - 3

    dump = formats.read_density(str(tmp_path / "density.0001.dat"), mode=2)
    got = dump["psi"].transpose(2, 1, 0).reshape(run.shape)
    assert np.array_equal(got, run.psi)
    run.close()

    # the reference's other files: the namelist echo the Fortran wrappers read
    # their cadence from, timec.dat, and the respar cuts of the start
    echo = tmp_path / "DFT4He3d.namelist.read"
    assert {k: he4gpu.read_namelist_int(echo, k) for k in ("iter0", "niter", "pener", "pcurr", "nx", "nz")} == \
        {"iter0": 0, "niter": niter, "pener": pener, "pcurr": pcurr, "nx": nx, "nz": nz}
    lines = (tmp_path / "timec.dat").read_text().splitlines()
    assert len(lines) == nz * (nx + 1)
    rows = np.array([[float(t) for t in ln.split()] for ln in lines if ln.strip()])
    tc = he4gpu.build_timec(cfg)[:, ny // 2, :]  # (z, x) at iy = ny/2 + 1
    assert np.array_equal(rows[:, 2].astype(np.float32), tc.reshape(-1))
    hx, hz = 2 * xmax / nx, 2 * zmax / nz
    np.testing.assert_allclose(rows[:nx, 0], -xmax + hx * np.arange(nx), rtol=0, atol=1e-12)
    np.testing.assert_allclose(rows[::nx, 1], -zmax + hz * np.arange(nz), rtol=0, atol=1e-12)
    first = he4gpu.Run(cfg, selec="Xe_He", r_cutoff=2.55, umax=2793.9365463, device_tables=True)
    first.set_state(psi, r, v)
    for name, field in (("hedenini", first.den), ("uimp", first.field("uimp"))):
        cx, cy, cz = nx // 2, ny // 2, nz // 2
        for ax, line in (("x", field[cz, cy, :]), ("y", field[cz, :, cx]), ("z", field[:, cy, cx])):
            cut = np.loadtxt(tmp_path / f"{name}-{ax}.dat")
            assert cut.shape == (len(line), 2)
            want = np.where(np.abs(line) < 1e-40, 0.0, line)
            np.testing.assert_allclose(cut[:, 1], want, rtol=1e-5, atol=0)
    first.close()
