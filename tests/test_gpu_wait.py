"""GPU: failure detection without a GPU fault. The bounded wait that every
TMA-fed kernel uses gives up on a barrier that nothing completes; the host
reads EGX_ERR_TIMEOUT, and the same context keeps working (an operator
apply after it still matches the oracle)."""
import os
import time

import numpy as np
import pytest

from extreme_gb300 import egx
from extreme_gb300.model import OmegaModel
from oracle import operator as op

pytestmark = pytest.mark.gpu


def test_bounded_wait_times_out_and_context_survives(egx_ctx):
    for limit in (50.0, 200.0):
        t = time.perf_counter()
        rc, msg = egx_ctx.wait_selftest(limit)
        dt = time.perf_counter() - t
        assert rc == egx.ERR_TIMEOUT and "timed out" in msg
        assert limit / 1e3 <= dt < limit / 1e3 + 5.0
    from tests.golden.make_golden import tiny_model
    gold = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "tiny.npz"))
    m = tiny_model()
    om = OmegaModel.build(m, 1.0)
    G = {c: gold["oracle_G_" + c] for c in ("xx", "xy", "yy", "zz", "xz", "yz")}
    g = egx_ctx.green_upload(G, m.nx, m.ny, m.nz)
    egx_ctx.op_prepare(g, om.zeta, om.zeta0, m.layer_thickness, egx.OP_A)
    y = egx_ctx.op_apply(gold["x"])
    want = op.apply(G, om, gold["x"], op.OP_A)
    assert np.linalg.norm(y - want) / np.linalg.norm(want) < 1e-10
    g.free()


def test_wait_limit_is_checked(egx_ctx):
    with pytest.raises(egx.EgxError):
        egx_ctx._check(egx_ctx.lib.egx_wait_selftest(egx_ctx.h, 0.0))
