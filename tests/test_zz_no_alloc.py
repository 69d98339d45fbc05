"""GPU: egx_dot_products_static, the dot-product reduction that allocates no
device memory (for callers that cannot allocate where they call it, e.g. a
host whose device memory belongs to its own pool allocator, or code inside a
solver callback), against egx_dot_products on the same vectors.

This file is named to be collected last: the entry point shares one static
device array across calls, so these checks also run after every other test
has used the library in the same process. Tolerance: 1e-12 relative per
column (the two kernels sum in different orders).
"""
import numpy as np
import pytest

from extreme_gb300 import egx

pytestmark = pytest.mark.gpu


def _case(rng, n, ncols):
    V = rng.standard_normal((n, ncols)) + 1j * rng.standard_normal((n, ncols))
    w = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    return V, w


def _static(ctx, V, w):
    import torch
    dev = torch.device("cuda", 0)
    Vt = torch.from_numpy(np.ascontiguousarray(V.T).view(np.float64).reshape(-1)).to(dev)
    wd = torch.from_numpy(np.ascontiguousarray(w).view(np.float64)).to(dev)
    out = torch.zeros(2 * V.shape[1], dtype=torch.float64, device=dev)
    torch.cuda.synchronize(dev)
    ctx.dot_products_static(Vt.data_ptr(), V.shape[1], wd.data_ptr(), V.shape[0], out.data_ptr())
    return out.cpu().numpy().view(np.complex128)


def test_static_dot_products_match_the_allocating_entry_point(egx_ctx):
    pytest.importorskip("torch")
    rng = np.random.default_rng(11)
    # two calls in a row with different sizes: the second must not see the first's partials
    for n, ncols in ((300001, 7), (4099, 3), (1, 1), (70000, 64)):
        V, w = _case(rng, n, ncols)
        want = egx_ctx.dot_products(V, w)
        got = _static(egx_ctx, V, w)
        np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-12 * np.abs(want).max())
        np.testing.assert_allclose(got, V.conj().T @ w, rtol=1e-10)


def test_static_dot_products_reject_more_columns_than_the_scratch_holds(egx_ctx):
    pytest.importorskip("torch")
    import torch
    dev = torch.device("cuda", 0)
    buf = torch.zeros(2 * 65 * 8, dtype=torch.float64, device=dev)
    with pytest.raises(egx.EgxError) as e:
        egx_ctx.dot_products_static(buf.data_ptr(), 65, buf.data_ptr(), 8, buf.data_ptr())
    assert e.value.code == egx.ERR_INVALID
    assert "64" in str(e.value)
