"""GPU: the learned preconditioner's network (egx_net_*) against the numpy
oracle -- forward, loss and every parameter block of the gradient (BF16
tensor-core GEMMs with FP32 accumulation against FP64) -- the identity of an
untrained network, Adam lowering the loss, and the mixed solve with the
network as its flexible preconditioner reaching the 1e-6 target."""
import numpy as np
import pytest

from oracle import spectral_net as sn

pytestmark = pytest.mark.gpu

# BF16 operands (8-bit significand), FP32 accumulation: normwise relative
# error per parameter block against the FP64 oracle
GRAD_TOL = 5e-2
LOSS_TOL = 2e-2
APPLY_TOL = 3e-2


@pytest.fixture(scope="module")
def ctx():
    from extreme_gb300 import egx
    c = egx.Context(0)
    yield c
    c.close()


def _net(ctx, nx, ny, nz, W, L, seed):
    from extreme_gb300 import egx
    net = egx.SpectralNet(ctx, nx, ny, nz, width=W, layers=L, seed=seed)
    rng = np.random.default_rng(seed)
    flat = net.params()
    lay, size = sn.layout(nz, W, L)
    assert size == net.size
    # nonzero output layer and biases, so that every block carries gradient
    for name in ("Q", "bQ", "bP") + tuple("b%d" % l for l in range(L)):
        off, shape = lay[name]
        k = int(np.prod(shape))
        flat[off:off + k] = 0.2 * rng.standard_normal(k)
    net.params(flat)
    return net, flat.astype(np.float64), lay


def _inputs(nx, ny, nz, B, seed):
    rng = np.random.default_rng(seed + 100)
    n = nx * ny * 3 * nz
    v = (rng.standard_normal((B, n)) + 1j * rng.standard_normal((B, n))).astype(np.complex64)
    t = (0.3 * (rng.standard_normal((B, n)) + 1j * rng.standard_normal((B, n)))).astype(np.complex64)
    logsig = rng.uniform(-3, 1, (nx, ny, nz)).astype(np.float32)
    return v, t, logsig


@pytest.mark.parametrize("nx,ny,nz,W,L,B,models", [(12, 10, 2, 16, 2, 2, 1), (32, 24, 4, 32, 3, 3, 1),
                                                   (16, 12, 5, 32, 4, 4, 4)])
def test_loss_and_gradient_match_oracle(ctx, nx, ny, nz, W, L, B, models):
    net, flat, lay = _net(ctx, nx, ny, nz, W, L, seed=nx)
    try:
        v, t, logsig = _inputs(nx, ny, nz, B, seed=nx)
        if models > 1:  # one conductivity model per sample (training batches across solves)
            rng = np.random.default_rng(nx + 7)
            logsig = rng.uniform(-3, 1, (models, nx, ny, nz)).astype(np.float32)
        net.set_model(logsig)
        loss, g = net.loss_grad(v, t, want_grad=True)
        ref_loss, ref_g = sn.loss_grad(flat, v.astype(np.complex128), t.astype(np.complex128),
                                       logsig.astype(np.float64), nx, ny, nz, W, L)
        assert abs(loss - ref_loss) <= LOSS_TOL * ref_loss, (loss, ref_loss)
        for name, (off, shape) in lay.items():
            k = int(np.prod(shape))
            a, b = g[off:off + k].astype(np.float64), ref_g[off:off + k]
            err = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)
            assert err <= GRAD_TOL, (name, err)
    finally:
        net.free()


def test_apply_matches_oracle(ctx):
    nx, ny, nz, W, L, B = 20, 16, 3, 16, 2, 2
    net, flat, _ = _net(ctx, nx, ny, nz, W, L, seed=5)
    try:
        v, _, logsig = _inputs(nx, ny, nz, B, seed=5)
        net.set_model(logsig)
        z = net.apply(v)
        ref = sn.apply(flat, v.astype(np.complex128), logsig.astype(np.float64), nx, ny, nz, W, L)
        err = np.linalg.norm(z - ref) / np.linalg.norm(ref - v)
        assert err <= APPLY_TOL, err
    finally:
        net.free()


def test_untrained_network_is_identity(ctx):
    from extreme_gb300 import egx
    nx, ny, nz = 16, 16, 2
    net = egx.SpectralNet(ctx, nx, ny, nz, width=16, layers=2, seed=1)
    try:
        v, _, logsig = _inputs(nx, ny, nz, 2, seed=1)
        net.set_model(logsig)
        np.testing.assert_array_equal(net.apply(v), v)
    finally:
        net.free()


def test_adam_lowers_the_loss(ctx):
    """A learnable target (a fixed lateral smoothing of v, scaled per layer):
    60 Adam steps on one batch lower the loss well below its start."""
    from extreme_gb300 import egx
    nx, ny, nz, B = 16, 16, 2, 4
    net = egx.SpectralNet(ctx, nx, ny, nz, width=16, layers=2, seed=3)
    try:
        v, _, logsig = _inputs(nx, ny, nz, B, seed=3)
        vv = v.reshape(B, nx, ny, 3, nz)
        t = 0.5 * (vv + np.roll(vv, 1, 1) + np.roll(vv, 1, 2)) / 3.0
        t = t.reshape(B, -1).astype(np.complex64)
        net.set_model(logsig)
        first = net.loss_grad(v, t)
        for _ in range(60):
            net.loss_grad(v, t)
            net.adam(3e-3)
        last = net.loss_grad(v, t)
        assert first > 0.9 and last < 0.5 * first, (first, last)
    finally:
        net.free()


def test_net_arguments_are_checked(ctx):
    from extreme_gb300 import egx
    with pytest.raises(egx.EgxError):
        egx.SpectralNet(ctx, 1, 8, 2)
    net = egx.SpectralNet(ctx, 8, 8, 2, width=8, layers=1)
    try:
        v = np.zeros((1, net.n), np.complex64)
        with pytest.raises(egx.EgxError):   # no model set yet
            net.apply(v)
        net.set_model(np.zeros((8, 8, 2), np.float32))
        with pytest.raises(egx.EgxError):
            net.apply(np.zeros((65, net.n), np.complex64))
        np.testing.assert_array_equal(net.apply(v), v)  # zero vector: rms 0, z = v
    finally:
        net.free()


def test_mixed_solve_with_learned_preconditioner(ctx):
    """Pairs (Arnoldi vector, GMRES(10) preconditioner output) from the
    solver on one model, a short training run that lowers their loss, then
    the mixed solve of a held-out model with the network as the flexible
    preconditioner: whatever the network's quality, the solve reaches the
    1e-6 target (the GMRES preconditioner takes over for an inner solve the
    network does not finish in four cycles), and the reference's method is
    unchanged beside it.

    No gain is asserted, because none was measured: trained on 2,000
    seeded 128x128x32 solves, the network predicts 32 % of the held-out
    correction energy (held-out loss 0.68), too little to converge within
    its four-cycle budget, so the held-out solves fall back and cost the
    budget on top of the GMRES-preconditioned applies (247 against 123 at
    0.01 Hz). What is asserted is that bound: the learned form never costs
    more than the budget plus the reference method."""
    from extreme_gb300 import egx, learned
    from extreme_gb300.model import scaled_model
    nx, ny, nz = 24, 24, 4
    f = 1.0
    sets = [learned.collect_pairs(ctx, scaled_model(nx, ny, nz, seed=11), f, n_vectors=3)]
    assert sets[0].v.shape == (6, nx * ny * 3 * nz)
    net = egx.SpectralNet(ctx, nx, ny, nz, width=16, layers=2, seed=0)
    try:
        before = learned.mean_loss(net, sets)
        log = learned.train(net, sets, steps=60, batch=4, lr=1e-3)
        assert np.isfinite(log.losses).all()
        assert learned.mean_loss(net, sets) < before
        rows = learned.evaluate(ctx, net, scaled_model(nx, ny, nz, seed=12), f)
        by = {r.method: r for r in rows}
        for m in ("gmres", "learned"):
            assert max(by[m].true_be) < 1e-6, (m, by[m].true_be)
        assert by["learned"].learned_uses >= 1
        assert by["gmres"].learned_uses == 0
        # four FGMRES(30) cycles of the network (one residual apply each),
        # then the GMRES-preconditioned solve
        budget = 4 * (30 + 1)
        assert by["learned"].applies[0] <= by["gmres"].applies[0] + budget + 2, (by["learned"].applies,
                                                                                   by["gmres"].applies)
        print("outer iterations gmres %d none %d learned %d (fallbacks %d)" % (
            by["gmres"].iterations[0], by["none"].iterations[0], by["learned"].iterations[0],
            by["learned"].fallbacks))
    finally:
        net.free()


def test_learned_net_must_match_the_grid(ctx):
    from extreme_gb300 import egx
    from extreme_gb300.forward import MixedSettings, Mt3DForwardSolver
    from extreme_gb300.model import scaled_model
    m = scaled_model(16, 16, 2, seed=3)
    net = egx.SpectralNet(ctx, 16, 12, 2, width=8, layers=1)
    try:
        net.set_model(np.zeros((16, 12, 2), np.float32))
        ctx.set_learned(net)
        solver = Mt3DForwardSolver(precision=egx.PREC_MIXED, mixed=MixedSettings(tol=1e-6), ctx=ctx)
        with pytest.raises(egx.EgxError):
            solver.solve(m, 1.0)
    finally:
        ctx.set_learned(None)
        net.free()


def test_tcgen05_pointwise_gemms_match_the_warp_level_kernel(ctx):
    """The network's pointwise GEMMs on the tcgen05 kernel (BF16 operands in
    shared memory, FP32 accumulator in tensor memory; the default) and on the
    warp-level mma.sync kernel round the same operands to BF16: loss, every
    gradient block and the apply agree to FP32 summation-order differences,
    and both stay within the BF16 bound of the FP64 oracle. The mesh has
    rows that do not fill the last 128-row tile."""
    nx, ny, nz, W, L, B = 18, 14, 5, 32, 3, 3
    net, flat, lay = _net(ctx, nx, ny, nz, W, L, seed=9)
    try:
        v, t, logsig = _inputs(nx, ny, nz, B, seed=9)
        net.set_model(logsig)
        out = {}
        for tc in (True, False):
            net.use_tcgen05(tc)
            loss, g = net.loss_grad(v, t, want_grad=True)
            out[tc] = (loss, g, net.apply(v))
        net.use_tcgen05(True)
        (l1, g1, z1), (l0, g0, z0) = out[True], out[False]
        assert abs(l1 - l0) <= 1e-4 * l0, (l1, l0)
        for name, (off, shape) in lay.items():
            k = int(np.prod(shape))
            a, b = g1[off:off + k], g0[off:off + k]
            assert np.linalg.norm(a - b) <= 1e-3 * max(np.linalg.norm(b), 1e-30), name
        assert np.linalg.norm(z1 - z0) <= 1e-4 * np.linalg.norm(z0 - v)
        ref_loss, _ = sn.loss_grad(flat, v.astype(np.complex128), t.astype(np.complex128),
                                   logsig.astype(np.float64), nx, ny, nz, W, L)
        assert abs(l1 - ref_loss) <= LOSS_TOL * ref_loss
    finally:
        net.free()
