"""he4g_get_psi_async / he4g_wait_psi through the C ABI: each call delivers
psi as it stood after the work issued before it, equal bit for bit to the
blocking he4g_get_psi, while later steps are already issued; in every
arithmetic form."""
import numpy as np
import pytest

from helpers import gpu_run, make_case

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", [0, 1, 2])
def test_async_reads_equal_blocking_reads(prec):
    torch = pytest.importorskip("torch")
    cfg, tk, psi, r, v, meta = make_case("he200_xe_40x48x64", precision=prec)
    a = gpu_run(cfg, tk, psi, r, v)
    b = gpu_run(cfg, tk, psi, r, v)
    n = cfg.nx * cfg.ny * cfg.nz
    bufs = [torch.empty(2 * n, dtype=torch.float64, pin_memory=True).numpy().view(np.complex128).reshape(a.shape)
            for _ in range(3)]
    want = []
    for k in range(3):
        a.step(2)
        a.get_psi_async(bufs[k])  # returns before the copy lands; the next steps are issued behind it
        b.step(2)
        want.append(b.psi)
    a.wait_psi()
    for k in range(3):
        assert np.array_equal(bufs[k], want[k]), k
    a.close()
    b.close()


def test_wait_without_a_copy_is_a_no_op():
    cfg, tk, psi, r, v, meta = make_case("he100_xe_32")
    a = gpu_run(cfg, tk, psi, r, v)
    a.wait_psi()
    out = np.empty(a.shape, dtype=np.complex128)
    a.get_psi_async(out)
    a.wait_psi()
    a.wait_psi()
    assert np.array_equal(out, a.psi)
    a.close()
