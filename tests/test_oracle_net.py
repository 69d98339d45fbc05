"""CPU: the oracle of the learned preconditioner's network. Its analytic
gradient equals central finite differences of its loss (FP64), every
parameter block; the untrained network (output layer zero) is the identity
preconditioner."""
import numpy as np

from oracle import spectral_net as sn


def _case(seed=0, nx=12, ny=10, nz=2, W=8, L=2, B=2):
    rng = np.random.default_rng(seed)
    _, size = sn.layout(nz, W, L)
    flat = 0.3 * rng.standard_normal(size)
    n = nx * ny * 3 * nz
    v = rng.standard_normal((B, n)) + 1j * rng.standard_normal((B, n))
    t = rng.standard_normal((B, n)) + 1j * rng.standard_normal((B, n))
    logsig = rng.uniform(-3, 1, (nx, ny, nz))
    return flat, v, t, logsig, (nx, ny, nz, W, L)


def test_gradient_matches_finite_differences():
    flat, v, t, logsig, dims = _case()
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
