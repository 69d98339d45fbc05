"""GPU: egx_dot_products_static, the dot-product reduction that allocates no
device memory, against egx_dot_products on the same vectors.

Who needs it: a caller that cannot allocate device memory at the point of
the call -- a host whose device memory belongs to its own pool allocator, or
a host function that a host-driven Krylov loop calls between its launches,
where a cudaMalloc would fail or stall the whole device mid-solve.

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


def _device(V, w):
    import torch
    dev = torch.device("cuda", 0)
    Vt = torch.from_numpy(np.ascontiguousarray(V.T).view(np.float64).reshape(-1)).to(dev)
    wd = torch.from_numpy(np.ascontiguousarray(w).view(np.float64)).to(dev)
    out = torch.zeros(2 * V.shape[1], dtype=torch.float64, device=dev)
    torch.cuda.synchronize(dev)
    return Vt, wd, out


def _static(ctx, V, w):
    Vt, wd, out = _device(V, w)
    ctx.dot_products_static(Vt.data_ptr(), V.shape[1], wd.data_ptr(), V.shape[0], out.data_ptr())
    return out.cpu().numpy().view(np.complex128)


def test_static_dot_products_match_the_allocating_entry_point(egx_ctx):
    pytest.importorskip("torch")
    rng = np.random.default_rng(11)
    # calls in a row with different sizes: a later call must not see an earlier one's partials
    for n, ncols in ((300001, 7), (4099, 3), (1, 1), (70000, 64)):
        V, w = _case(rng, n, ncols)
        want = egx_ctx.dot_products(V, w)
        got = _static(egx_ctx, V, w)
        np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-12 * np.abs(want).max())
        np.testing.assert_allclose(got, V.conj().T @ w, rtol=1e-10)


def test_static_dot_products_allocate_nothing():
    """On a context that has never allocated its own scratch, two calls in a
    row leave the library's device-allocation count unchanged, while the
    allocating entry point on another fresh context does allocate."""
    pytest.importorskip("torch")
    rng = np.random.default_rng(12)
    V, w = _case(rng, 50001, 9)
    Vt, wd, out = _device(V, w)
    ctx = egx.Context(0)
    try:
        before = egx.Context.device_allocations()
        for _ in range(2):
            ctx.dot_products_static(Vt.data_ptr(), V.shape[1], wd.data_ptr(), V.shape[0], out.data_ptr())
        assert egx.Context.device_allocations() == before
        got = out.cpu().numpy().view(np.complex128)
        np.testing.assert_allclose(got, V.conj().T @ w, rtol=1e-10)
    finally:
        ctx.close()
    other = egx.Context(0)
    try:
        before = egx.Context.device_allocations()
        other.dot_products(V, w)
        assert egx.Context.device_allocations() > before
    finally:
        other.close()


def test_static_dot_products_reject_more_columns_than_the_scratch_holds(egx_ctx):
    pytest.importorskip("torch")
    import torch
    dev = torch.device("cuda", 0)
    buf = torch.zeros(2 * 65 * 8, dtype=torch.float64, device=dev)
    with pytest.raises(egx.EgxError) as e:
        egx_ctx.dot_products_static(buf.data_ptr(), 65, buf.data_ptr(), 8, buf.data_ptr())
    assert e.value.code == egx.ERR_INVALID
    assert "64" in str(e.value)


def test_static_dot_products_reject_misaligned_pointers(egx_ctx):
    """An 8-byte offset pointer is rejected on the host; nothing is launched."""
    pytest.importorskip("torch")
    import torch
    dev = torch.device("cuda", 0)
    buf = torch.zeros(2 * 4 * 16 + 2, dtype=torch.float64, device=dev)
    base = buf.data_ptr()
    launches = egx_ctx.launch_count()
    for v_off, w_off, o_off in ((8, 0, 0), (0, 8, 0), (0, 0, 8)):
        with pytest.raises(egx.EgxError) as e:
            egx_ctx.dot_products_static(base + v_off, 2, base + 512 + w_off, 8, base + 768 + o_off)
        assert e.value.code == egx.ERR_INVALID
        assert "aligned" in str(e.value)
    assert egx_ctx.launch_count() == launches
