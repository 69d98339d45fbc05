"""CPU: the oracle of the learned preconditioner's network. Its analytic
gradient equals central finite differences of its loss (FP64), every
parameter block (one conductivity model for all samples, or one per
sample); the untrained network (output layer zero) is the identity
preconditioner; the encoding maps the anomaly layout to (x, y, z, channel)
and back."""
import numpy as np
import pytest

from oracle import spectral_net as sn


def _case(seed=0, nx=12, ny=10, nz=3, W=8, L=2, B=2, models=1):
    rng = np.random.default_rng(seed)
    _, size = sn.layout(nz, W, L)
    flat = 0.3 * rng.standard_normal(size)
    n = nx * ny * 3 * nz
    v = rng.standard_normal((B, n)) + 1j * rng.standard_normal((B, n))
    t = rng.standard_normal((B, n)) + 1j * rng.standard_normal((B, n))
    logsig = rng.uniform(-3, 1, (nx, ny, nz) if models == 1 else (models, nx, ny, nz))
    return flat, v, t, logsig, (nx, ny, nz, W, L)


@pytest.mark.parametrize("models", [1, 2])
def test_gradient_matches_finite_differences(models):
    flat, v, t, logsig, dims = _case(models=models)
    loss, g = sn.loss_grad(flat, v, t, logsig, *dims)
    lay, _ = sn.layout(dims[2], dims[3], dims[4])
    rng = np.random.default_rng(1)
    h = 1e-6
    for name, (off, shape) in lay.items():
        size = int(np.prod(shape))
        for idx in rng.choice(size, min(4, size), replace=False):
            k = off + idx
            fp, fm = flat.copy(), flat.copy()
            fp[k] += h
            fm[k] -= h
            num = (sn.loss_grad(fp, v, t, logsig, *dims)[0] - sn.loss_grad(fm, v, t, logsig, *dims)[0]) / (2 * h)
            assert abs(num - g[k]) <= 1e-6 * max(1.0, abs(num)), (name, idx, num, g[k])


def test_untrained_network_is_identity():
    flat, v, t, logsig, dims = _case()
    lay, _ = sn.layout(dims[2], dims[3], dims[4])
    for name in ("Q", "bQ"):
        off, shape = lay[name]
        flat[off:off + int(np.prod(shape))] = 0
    z = sn.apply(flat, v, logsig, *dims)
    np.testing.assert_array_equal(z, v)


def test_encoding_round_trip():
    """X0's six field channels and the output decoding are inverse maps of
    the anomaly layout ((x ny + y) 3 + c) nz + z."""
    nx, ny, nz = 5, 4, 3
    rng = np.random.default_rng(3)
    v = rng.standard_normal((2, nx * ny * 3 * nz)) + 1j * rng.standard_normal((2, nx * ny * 3 * nz))
    X0, rms, inv = sn.encode(v, np.zeros((nx, ny, nz)), nx, ny, nz)
    # element (x=1, y=2, c=1, z=2) of sample 1
    e = ((1 * ny + 2) * 3 + 1) * nz + 2
    assert np.isclose(X0[1, 1, 2, 2, 1], v[1, e].real * inv[1])
    assert np.isclose(X0[1, 1, 2, 2, 4], v[1, e].imag * inv[1])
    T = sn.target(v, inv, nx, ny, nz)
    back = (T[..., :3] + 1j * T[..., 3:]).transpose(0, 1, 2, 4, 3).reshape(2, -1) / inv[:, None]
    np.testing.assert_allclose(back, v, rtol=1e-14)
