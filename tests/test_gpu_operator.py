"""GPU: the FFT and the CIE operator through the C ABI against the oracle.

Tolerances: complex128 path <= 1e-10 relative (2-norm), the bar the
reference's operator apply is held to; complex64 path <= 2e-5 relative.
"""
import os

import numpy as np
import pytest

from extreme_gb300 import egx
from extreme_gb300.model import OmegaModel, small_model
from oracle import green
from oracle import operator as op

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "tiny.npz")
COMPS = ("xx", "xy", "yy", "zz", "xz", "yz")


def rel(a, b):
    return np.linalg.norm(np.ravel(a) - np.ravel(b)) / np.linalg.norm(np.ravel(b))


@pytest.mark.parametrize("shape", [(64, 64, 24), (16, 12, 5), (14, 10, 7), (12, 18, 3), (8, 8, 1)])
@pytest.mark.parametrize("sign", [-1, 1])
def test_fft2d_matches_numpy(egx_ctx, shape, sign):
    rng = np.random.default_rng(1)
    a = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    want = np.fft.fft2(a, axes=(0, 1)) if sign < 0 else np.fft.ifft2(a, axes=(0, 1)) * (shape[0] * shape[1])
    got = egx_ctx.fft2d(a.copy(), sign)
    assert rel(got, want) < 1e-13


def _tiny():
    from tests.golden.make_golden import tiny_model
    m = tiny_model()
    return m, OmegaModel.build(m, 1.0)


@pytest.mark.parametrize("op_type", [op.OP_A, op.OP_CHI0])
def test_apply_tiny_golden(egx_ctx, op_type):
    gold = np.load(GOLD)
    m, om = _tiny()
    G = {c: gold["oracle_G_" + c] for c in COMPS}
    g = egx_ctx.green_upload(G, m.nx, m.ny, m.nz)
    egx_ctx.op_prepare(g, om.zeta, om.zeta0, m.layer_thickness, op_type)
    y = egx_ctx.op_apply(gold["x"])
    want = gold["oracle_apply_A"] if op_type == op.OP_A else gold["oracle_apply_chi0"]
    assert rel(y, want) < 1e-10
    g.free()


@pytest.fixture(scope="module")
def small_case():
    m = small_model()
    om = OmegaModel.build(m, 0.1)
    G = green.green_tensor(om, 10)
    return m, om, G


def test_green_roundtrip_download(egx_ctx, small_case):
    m, om, G = small_case
    g = egx_ctx.green_upload(G, m.nx, m.ny, m.nz)
    back = g.download()
    for c in COMPS:
        assert rel(back[c], G[c]) < 1e-12, c
    g.free()


@pytest.mark.parametrize("op_type", [op.OP_A, op.OP_CHI0])
def test_apply_small_matches_oracle(egx_ctx, small_case, op_type):
    m, om, G = small_case
    g = egx_ctx.green_upload(G, m.nx, m.ny, m.nz, precision=egx.PREC_MIXED)
    egx_ctx.op_prepare(g, om.zeta, om.zeta0, m.layer_thickness, op_type)
    rng = np.random.default_rng(2)
    n = m.nx * m.ny * 3 * m.nz
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    want = op.apply(G, om, x, op_type)
    y = egx_ctx.op_apply(x)
    assert rel(y, want) < 1e-10
    # two right-hand sides in one apply
    x2 = np.concatenate([x, 1j * x[::-1]])
    y2 = egx_ctx.op_apply(x2, nrhs=2)
    assert rel(y2[:n], want) < 1e-10
    assert rel(y2[n:], op.apply(G, om, 1j * x[::-1], op_type)) < 1e-10
    # complex64 operator
    y32 = egx_ctx.op_apply_c64(x.astype(np.complex64))
    assert rel(y32, want) < 2e-5
    g.free()


@pytest.mark.parametrize("variant", [0, 1, 2])
@pytest.mark.parametrize("nz", [16, 32, 48])
def test_c64_subblock_apply_matches_oracle(egx_ctx, nz, variant):
    """complex64 apply on the sub-block Green layout (nz in {16, 32, 48}),
    one to three right-hand sides (passes of two and one), ragged edges
    (nx != ny, the kx = 0, nx and ky = 0, ny points with fewer mirrors),
    with the two-source passes on the built-in FP16-split kernel by role
    (variant 0), the TF32-split (variant 1) and the FP16-split lockstep
    (variant 2) tensor-core kernels."""
    from extreme_gb300.model import freq_to_omega, scaled_model
    m = scaled_model(10, 6, nz, seed=3)
    f = m.frequencies[2]
    om = OmegaModel.build(m, f)
    g = egx_ctx.green_build(m, freq_to_omega(f), 10, egx.PREC_MIXED)
    G = g.download()
    egx_ctx.op_prepare(g, om.zeta, om.zeta0, m.layer_thickness, op.OP_A)
    rng = np.random.default_rng(nz)
    n = m.nx * m.ny * 3 * m.nz
    xs = rng.standard_normal((3, n)) + 1j * rng.standard_normal((3, n))
    want = [op.apply(G, om, xs[i], op.OP_A) for i in range(3)]
    egx_ctx.apply_variant(0, variant)
    try:
        for nrhs in (1, 2, 3):
            y = egx_ctx.op_apply_c64(xs[:nrhs].reshape(-1).astype(np.complex64), nrhs=nrhs)
            for i in range(nrhs):
                assert rel(y[i * n:(i + 1) * n], want[i]) < 2e-5, (nrhs, i)
    finally:
        egx_ctx.apply_variant(0, 0)
        g.free()


@pytest.mark.parametrize("nz,nrhs", [(48, 2), (48, 1), (7, 3), (2, 10)])
def test_double_fp32_apply_matches_complex128(egx_ctx, nz, nrhs):
    """The mixed form's residual apply (contraction as Dot2 on float pairs)
    against the complex128 apply: <= 1e-12 relative per vector, ragged
    edges (nx != ny), one to ten right-hand sides (passes of eight points)."""
    from extreme_gb300.model import freq_to_omega, scaled_model
    m = scaled_model(10, 6, nz, seed=5)
    f = m.frequencies[1]
    om = OmegaModel.build(m, f)
    g = egx_ctx.green_build(m, freq_to_omega(f), 10, egx.PREC_MIXED)
    egx_ctx.op_prepare(g, om.zeta, om.zeta0, m.layer_thickness, op.OP_A)
    rng = np.random.default_rng(nz + nrhs)
    n = m.nx * m.ny * 3 * m.nz
    # magnitudes spread over many decades, as in a converged residual
    xs = (rng.standard_normal((nrhs, n)) + 1j * rng.standard_normal((nrhs, n))) * 10.0 ** rng.uniform(-8, 2, (nrhs, n))
    want = egx_ctx.op_apply(xs.reshape(-1), nrhs=nrhs)
    got = egx_ctx.op_apply_ds(xs.reshape(-1), nrhs=nrhs)
    for i in range(nrhs):
        assert rel(got[i * n:(i + 1) * n], want[i * n:(i + 1) * n]) < 1e-12, i
    g.free()


def test_apply_before_prepare_is_state_error():
    ctx = egx.Context(0)
    with pytest.raises(egx.EgxError) as e:
        ctx.op_apply(np.zeros(24, complex))
    assert e.value.code == egx.ERR_STATE
    ctx.close()


def test_c64_apply_512_point_lines_match_complex128(egx_ctx):
    """The complex64 apply with 512-point lines in both directions (the
    two-pass register FFT of 32 x 16 points) against the complex128 apply
    of the same operator (three-pass FFT) on the device, 256x256x16, two
    right-hand sides: complex64 accuracy."""
    from extreme_gb300.model import freq_to_omega, scaled_model
    m = scaled_model(256, 256, 16, seed=4)
    f = m.frequencies[1]
    om = OmegaModel.build(m, f)
    g = egx_ctx.green_build(m, freq_to_omega(f), 10, egx.PREC_MIXED)
    try:
        egx_ctx.op_prepare(g, om.zeta, om.zeta0, m.layer_thickness, op.OP_A)
        rng = np.random.default_rng(16)
        n = m.nx * m.ny * 3 * m.nz
        xs = rng.standard_normal((2, n)) + 1j * rng.standard_normal((2, n))
        y32 = egx_ctx.op_apply_c64(xs.reshape(-1).astype(np.complex64), nrhs=2)
        for i in range(2):
            y64 = egx_ctx.op_apply(xs[i])
            assert rel(y32[i * n:(i + 1) * n], y64) < 2e-6, i
    finally:
        g.free()
