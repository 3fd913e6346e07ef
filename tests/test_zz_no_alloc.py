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


def test_forceimp_noalloc_matches_forceimp():
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
    stream = torch.cuda.current_stream()
    for _ in range(2):
        out.fill_(float("nan"))
        rc = run.lib.he4g_forceimp_noalloc(C.c_void_p(den.data_ptr()), C.c_void_p(uimp.data_ptr()), cfg.nx,
                                           cfg.ny, cfg.nz, cfg.xmax, cfg.ymax, cfg.zmax,
                                           C.c_void_p(out.data_ptr()), C.c_void_p(stream.cuda_stream))
        assert rc == 0
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        np.testing.assert_allclose(got, F_ref, rtol=FIELD_TOL, atol=FIELD_TOL * np.max(np.abs(F_ref)))
    run.close()


def test_forceimp_noalloc_rejects_grids_beyond_its_scratch():
    """A grid that needs more partial-sum slots than the built-in array holds
    is refused before any device work."""
    from he4gpu import abi
    lib = abi.load()
    dummy = C.c_void_p(16)
    rc = lib.he4g_forceimp_noalloc(dummy, dummy, 1024, 1024, 1024, 10.0, 10.0, 10.0, dummy, None)
    assert rc == abi.HE4G_EINVAL
