"""GPU check of he4g_forceimp_noalloc, the impurity force for callers that
cannot allocate device memory: hosts that keep the fields in device arrays
they manage themselves and call the force inside their time loop, where
cudaMalloc would synchronise the whole device every step and can fail once
other runs sharing the GPU have filled its memory.

The entry point is called through the C ABI on device copies of a run's
density and impurity potential, twice in a row, and compared with
he4g_forceimp of the same run. This file is collected last, so a run that
stops at the first failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import gpu_run, make_case

pytestmark = pytest.mark.gpu

FIELD_TOL = 1e-12  # the tolerance of the single-evaluation parity tests


def _call(lib, den, uimp, n, ext, out, stream):
    return lib.he4g_forceimp_noalloc(C.c_void_p(den.data_ptr()), C.c_void_p(uimp.data_ptr()), n[0], n[1], n[2],
                                     ext[0], ext[1], ext[2], C.c_void_p(out.data_ptr()),
                                     C.c_void_p(stream) if stream is not None else None)


def test_forceimp_noalloc_matches_forceimp():
    """Two calls in a row on torch's stream, then one on the legacy default
    stream (NULL), each equal to he4g_forceimp; the device's free memory is
    the same before and after them. One round of the same operations comes
    before the memory is read: with lazy module loading, the first launch of
    a kernel (the library's, and torch's fill kernel here) loads its module
    into device memory, and the first call in a context looks up the scratch
    array."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    cfg, tk, psi, r, v, meta = make_case("he300_ar_48")
    run = gpu_run(cfg, tk, psi, r, v)
    run.step(4)  # 3 Runge-Kutta-Gill + 1 predictor-corrector step: a non-trivial state
    F_ref = run.forceimp()
    den = torch.from_numpy(run.den).to("cuda")
    uimp = torch.from_numpy(run.field("uimp")).to("cuda")
    out = torch.empty(3, dtype=torch.float64, device="cuda")
    n, ext = (cfg.nx, cfg.ny, cfg.nz), (cfg.xmax, cfg.ymax, cfg.zmax)
    stream = torch.cuda.current_stream().cuda_stream

    def calls():
        for s in (stream, stream, None):
            out.fill_(float("nan"))
            assert _call(run.lib, den, uimp, n, ext, out, s) == 0
            torch.cuda.synchronize()
            got = out.cpu().numpy()
            np.testing.assert_allclose(got, F_ref, rtol=FIELD_TOL, atol=FIELD_TOL * np.max(np.abs(F_ref)))

    calls()  # modules loaded, scratch address looked up
    free0, _ = torch.cuda.mem_get_info()
    calls()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, "device memory changed across the calls"
    run.close()


def _force_torch(den, uimp, h):
    """F = -sum(grad den * uimp) dV in PyTorch FP64: the 13-point first
    derivative (Fornberg coefficients, zero padding beyond the grid)."""
    import torch
    c = [6.0 / 7.0, -15.0 / 56.0, 5.0 / 63.0, -1.0 / 56.0, 1.0 / 385.0, -1.0 / 5544.0]
    nz, ny, nx = den.shape
    p = torch.nn.functional.pad(den, (6, 6, 6, 6, 6, 6))
    F, scale = [], []
    for ax, hh in ((2, h[0]), (1, h[1]), (0, h[2])):
        g = torch.zeros_like(den)
        for o in range(1, 7):
            sl_hi = [slice(6, 6 + nz), slice(6, 6 + ny), slice(6, 6 + nx)]
            sl_lo = list(sl_hi)
            sl_hi[ax] = slice(6 + o, 6 + o + den.shape[ax])
            sl_lo[ax] = slice(6 - o, 6 - o + den.shape[ax])
            g += c[o - 1] * (p[tuple(sl_hi)] - p[tuple(sl_lo)])
        t = g / hh * uimp
        F.append(-float(t.sum()) * h[0] * h[1] * h[2])
        scale.append(float(t.abs().sum()) * h[0] * h[1] * h[2])
    return np.array(F), np.array(scale)


def test_forceimp_noalloc_near_its_largest_grid():
    """320^3 (128000 of the 131072 partial-sum slots): two calls against a
    PyTorch FP64 evaluation of the same sum, within 1e-12 of the sum of the
    terms' magnitudes."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from he4gpu import abi
    lib = abi.load()
    n = 320
    xmax = 64.0
    h = (2 * xmax / n,) * 3
    ax = -xmax + h[0] * torch.arange(n, dtype=torch.float64, device="cuda")
    z, y, x = torch.meshgrid(ax, ax, ax, indexing="ij")
    den = 0.02 / (1.0 + torch.exp((torch.sqrt((x - 3.0) ** 2 + (y + 2.0) ** 2 + (z - 1.0) ** 2) - 30.0) / 0.8))
    uimp = 100.0 * torch.exp(-((x - 10.0) ** 2 + (y - 5.0) ** 2 + (z + 28.0) ** 2) / 20.0)
    del x, y, z
    F_ref, scale = _force_torch(den, uimp, h)
    assert np.all(np.abs(F_ref) > 1e-6 * scale)  # a force with all three components
    out = torch.empty(3, dtype=torch.float64, device="cuda")
    for _ in range(2):
        out.fill_(float("nan"))
        assert _call(lib, den, uimp, (n, n, n), (xmax, xmax, xmax), out,
                     torch.cuda.current_stream().cuda_stream) == 0
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        assert np.all(np.abs(got - F_ref) <= 1e-12 * scale), (got, F_ref, scale)


def test_forceimp_noalloc_rejects_grids_beyond_its_scratch():
    """A grid that needs more partial-sum slots than the built-in array holds
    is refused before any device work."""
    from he4gpu import abi
    lib = abi.load()
    dummy = C.c_void_p(16)
    rc = lib.he4g_forceimp_noalloc(dummy, dummy, 1024, 1024, 1024, 10.0, 10.0, 10.0, dummy, None)
    assert rc == abi.HE4G_EINVAL
    # 384^3 needs 6 * 96 * 384 = 221184 slots; and a zero or non-finite extent
    assert lib.he4g_forceimp_noalloc(dummy, dummy, 384, 384, 384, 10.0, 10.0, 10.0, dummy, None) == abi.HE4G_EINVAL
    for ext in ((0.0, 10.0, 10.0), (10.0, float("nan"), 10.0), (10.0, 10.0, float("inf"))):
        assert lib.he4g_forceimp_noalloc(dummy, dummy, 32, 32, 32, *ext, dummy, None) == abi.HE4G_EINVAL
