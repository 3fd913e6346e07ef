"""The reference's file formats: namelist input, readenc / printoutc density
and wave-function files (host-side, no GPU)."""
import numpy as np
import pytest

from he4gpu import formats

NAMELIST = """ &input
 Lambdah = 2.d0
 tzmean = 49.2d0
 tzsurf = 2.d0
 mimpur = 131.29d0
 title = '4He_1000 + Xe'
 n4 = 1000
 mode = 2
 selec = 'Xe_He'
 r_cutoff = 2.55d0
 umax = 2.7939365463E+03
 lselection = .true.
 filedenin  = 'den.in'
 nx = 64, ny = 64, nz = 80
 xmax = 25.6d0
 ymax = 25.6d0
 zmax = 32.d0
 core4='OT'
 lsolid = .true.
 ximp= -27.0d0
 vzimp = 2.d0
 deltatps = 1.d-4
 pener = 200
 /
"""


def test_namelist_values_and_run():
    nl = formats.read_namelist(NAMELIST)
    assert nl["lambdah"] == 2.0 and nl["tzmean"] == 49.2 and nl["n4"] == 1000
    assert nl["title"] == "4He_1000 + Xe" and nl["selec"] == "Xe_He" and nl["lselection"] is True
    assert nl["umax"] == pytest.approx(2793.9365463) and nl["nz"] == 80
    cfg, over, table, rimp, vimp, loop = formats.run_from_namelist(nl)
    assert cfg == dict(nx=64, ny=64, nz=80, xmax=25.6, ymax=25.6, zmax=32.0)
    assert over["lsolid"] == 1 and over["core"] == 0 and over["mimpur"] == 131.29
    assert over["deltat"] == pytest.approx(1e-4 / 7.63822291)
    assert table == dict(selec="Xe_He", r_cutoff=2.55, umax=pytest.approx(2793.9365463))
    assert rimp.tolist() == [-27.0, 0.0, 0.0]
    assert vimp[2] == pytest.approx(2.0 * 7.63822291)
    assert loop["pener"] == 200 and loop["mode"] == 2


def test_namelist_drives_a_config():
    import he4gpu
    cfg, over, table, rimp, vimp, loop = formats.run_from_namelist(formats.read_namelist(NAMELIST))
    c = he4gpu.default_config(cfg["nx"], cfg["ny"], cfg["nz"], cfg["xmax"], cfg["ymax"], cfg["zmax"], **over)
    assert (c.nx, c.ny, c.nz, c.lsolid, c.tzmean) == (64, 64, 80, 1, 49.2)


def test_write_then_read_is_exact(tmp_path):
    rng = np.random.default_rng(3)
    psi = (rng.standard_normal((6, 4, 5)) + 1j * rng.standard_normal((6, 4, 5))) * 1e-3
    psi[0, 0, 0] = 1e-300 + 0j  # tiny values survive too
    rimp, vimp = np.array([1.5, -2.25, 3.0]), np.array([0.0, 0.1, 22.9])
    p = tmp_path / "den.out"
    formats.write_density(p, psi, rimp, vimp, 4.8, 3.2, 4.0, iteration=7, dtps=1e-4, energies={"etot": -12.5})
    d = formats.read_density(p, mode=2)
    assert (d["nx"], d["ny"], d["nz"]) == (6, 4, 5)
    assert d["hx"] == pytest.approx(1.6) and d["zmax"] == 4.0
    assert np.array_equal(d["rimp"], rimp) and np.array_equal(d["vimp"], vimp)
    assert np.array_equal(d["psi"], psi)
    text = p.read_text().splitlines()
    assert text[1].startswith("#  Density after") and text[16].startswith("#  Etot") and "-1.25" in text[16]


def test_compiler_list_directed_output(tmp_path):
    # repeat counts, D exponents, records split over lines, parentheses with blanks
    body = ["# header", "#  ",
            " 2.0D0 2.0D0 2.0D0 1.0D0 1.0D0",
            " 1.0D0 3 3 1",
            " 0.5D0 0.0D0 -0.5D0",
            " 1.0D-1 2.0D-1 3.0D-1",
            " 5*(0.0D0,0.0D0) ( 1.5D0 , -2.0D-3 )",
            " 2*(1.0E0,1.0E0)",
            " (3.0,4.0)"]
    p = tmp_path / "listdirected.den"
    p.write_text("\n".join(body) + "\n")
    d = formats.read_density(p, mode=2)
    assert d["rimp"].tolist() == [0.5, 0.0, -0.5] and d["vimp"].tolist() == [0.1, 0.2, 0.3]
    flat = d["psi"].reshape(-1, order="F")
    assert flat.tolist() == [0j] * 5 + [1.5 - 2e-3j, 1 + 1j, 1 + 1j, 3 + 4j]


def test_mode0_density_and_mode3_invariants(tmp_path):
    p0 = tmp_path / "m0.den"
    p0.write_text("# a density\n 1.0 1.0 1.0 1.0 1.0 1.0 2 1 1 T -3.0 0.0 0.0\n 0.25 0.5\n")
    d0 = formats.read_density(p0, mode=0)
    assert d0["limp"] is True and d0["rimp"].tolist() == [-3.0, 0.0, 0.0]
    assert d0["den"].reshape(-1).tolist() == [0.25, 0.5]
    p3 = tmp_path / "m3.den"
    p3.write_text("#\n 1 1 1 1 1 1 1 1 2\n 0 0 0\n 0 0 0\n 2\n (1,0) (0,1)\n (2,0) (0,2)\n")
    d3 = formats.read_density(p3, mode=3)
    assert d3["invar"].tolist() == [1 + 0j, 1j] and d3["psi"].reshape(-1).tolist() == [2 + 0j, 2j]
