"""GPU: the FP64 anomaly-to-anomaly Green tensor built on the device against
the oracle (per component, <= 1e-10 relative in the 2-norm) and the
operator built from it. The mixed form's tensor (FP64 recursions, Hankel
sums and face integrals, complex64 lateral FFT) is within 1e-6 of it."""
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


def test_green_build_tiny_matches_golden(egx_ctx):
    from tests.golden.make_golden import tiny_model
    gold = np.load(GOLD)
    m = tiny_model()
    g = egx_ctx.green_build(m, OmegaModel.build(m, 1.0).omega, n_hankels=4)
    G = g.download()
    for c in COMPS:
        assert rel(G[c], gold["oracle_G_" + c]) < 1e-10, c
    g.free()


@pytest.mark.parametrize("freq", [0.1, 10.0])
def test_green_build_small_matches_oracle(egx_ctx, freq):
    m = small_model()
    om = OmegaModel.build(m, freq)
    want = green.green_tensor(om, 10)
    g = egx_ctx.green_build(m, om.omega, n_hankels=10)
    G = g.download()
    for c in COMPS:
        assert rel(G[c], want[c]) < 1e-10, (c, rel(G[c], want[c]))
    # and the operator built on it
    egx_ctx.op_prepare(g, om.zeta, om.zeta0, m.layer_thickness, op.OP_A)
    rng = np.random.default_rng(4)
    n = m.nx * m.ny * 3 * m.nz
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    assert rel(egx_ctx.op_apply(x), op.apply(want, om, x, op.OP_A)) < 1e-10
    g.free()


@pytest.mark.parametrize("freq", [0.1, 10.0])
def test_mixed_green_lateral_fft32(egx_ctx, freq):
    m = small_model()
    om = OmegaModel.build(m, freq)
    g64 = egx_ctx.green_build(m, om.omega, n_hankels=10)
    g32 = egx_ctx.green_build(m, om.omega, 10, egx.PREC_MIXED)
    A, B = g64.download(), g32.download()
    for c in COMPS:
        err = rel(B[c], A[c])
        assert 1e-12 < err < 1e-6, (c, err)   # complex64 transform: not bit-equal, within single precision
    g64.free()
    g32.free()


def test_green_build_rejects_straddling_layer(egx_ctx):
    m = small_model()
    m.layer_depth = m.layer_depth + 100.0  # 1.1-3.1 km: layer 3 crosses the 2 km interface
    with pytest.raises(egx.EgxError) as e:
        egx_ctx.green_build(m, 1.0, n_hankels=10)
    assert e.value.code == egx.ERR_MODEL
