"""GPU: FGMRES with the GMRES preconditioner and the mixed-precision solve
through the C ABI against the oracle.

The complex128 solve must reproduce the oracle's iteration count and its
solution to within 10x the FGMRES tolerance; the mixed solve must reach its
target true residual and stay within 1e-5 (relative) of the complex128
solution.
"""
import os

import numpy as np
import pytest

from extreme_gb300 import egx
from extreme_gb300.model import OmegaModel, small_model
from oracle import fgmres, green, mt
from oracle import operator as op

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "tiny.npz")
COMPS = ("xx", "xy", "yy", "zz", "xz", "yz")


def rel(a, b):
    return np.linalg.norm(np.ravel(a) - np.ravel(b)) / np.linalg.norm(np.ravel(b))


def test_fgmres_tiny_matches_golden(egx_ctx):
    from tests.golden.make_golden import tiny_model
    gold = np.load(GOLD)
    m = tiny_model()
    om = OmegaModel.build(m, 1.0)
    G = {c: gold["oracle_G_" + c] for c in COMPS}
    g = egx_ctx.green_upload(G, m.nx, m.ny, m.nz)
    egx_ctx.op_prepare(g, om.zeta, om.zeta0, m.layer_thickness, op.OP_A)
    b = gold["oracle_apply_chi0"]
    x, r = egx_ctx.fgmres_solve(b, b, m_out=5, m_in=3, tol=1e-9, max_restarts=50)
    assert r["converged"]
    assert r["iterations"] == int(gold["oracle_solve_iterations"])
    assert r["n_applies"] == int(gold["oracle_solve_applies"])
    assert rel(x, gold["oracle_solve_x"]) < 1e-8
    g.free()


@pytest.fixture(scope="module")
def small_solve():
    m = small_model()
    om = OmegaModel.build(m, 0.1)
    G = green.green_tensor(om, 10)
    out = mt.solve_polarization(om, G, "x", m_out=20, m_in=10, tol=1e-8)
    return m, om, G, out


def test_fgmres_small_matches_oracle(egx_ctx, small_solve):
    m, om, G, out = small_solve
    g = egx_ctx.green_upload(G, m.nx, m.ny, m.nz)
    egx_ctx.op_prepare(g, om.zeta, om.zeta0, m.layer_thickness, op.OP_CHI0)
    chi0 = egx_ctx.op_apply(out.js)
    assert rel(chi0, out.chi0) < 1e-10
    egx_ctx.op_prepare(g, om.zeta, om.zeta0, m.layer_thickness, op.OP_A)
    x, r = egx_ctx.fgmres_solve(chi0, chi0, m_out=20, m_in=10, tol=1e-8, max_restarts=100)
    assert r["converged"]
    assert r["iterations"] == out.result.iterations
    assert rel(x, out.chi) < 10 * 1e-8
    g.free()


def test_nonconvergence_returns_status(egx_ctx, small_solve):
    m, om, G, out = small_solve
    g = egx_ctx.green_upload(G, m.nx, m.ny, m.nz)
    egx_ctx.op_prepare(g, om.zeta, om.zeta0, m.layer_thickness, op.OP_A)
    x, r = egx_ctx.fgmres_solve(out.chi0, out.chi0, m_out=2, m_in=1, tol=1e-14, max_restarts=2)
    assert not r["converged"]
    with pytest.raises(egx.EgxError) as e:
        egx_ctx.fgmres_solve(out.chi0, out.chi0, m_out=2, m_in=1, tol=1e-14, max_restarts=2,
                             raise_on_nonconv=True)
    assert e.value.code == egx.ERR_NOT_CONVERGED
    g.free()


def test_mixed_solve_small(egx_ctx, small_solve):
    m, om, G, out = small_solve
    g = egx_ctx.green_upload(G, m.nx, m.ny, m.nz, precision=egx.PREC_MIXED)
    egx_ctx.op_prepare(g, om.zeta, om.zeta0, m.layer_thickness, op.OP_A)
    x, r = egx_ctx.mixed_solve(out.chi0, np.zeros_like(out.chi0), tol=1e-6, inner_tol=1e-4)
    assert r["converged"], r
    assert r["true_be"] < 1e-6
    # verify the true residual with the oracle operator
    A = op.Operator(G, om, op.OP_A)
    res = np.linalg.norm(out.chi0 - A(x)) / np.linalg.norm(out.chi0)
    assert res < 1e-6
    assert rel(x, out.chi) < 1e-5
    g.free()


@pytest.mark.parametrize("precision", [egx.PREC_FP64, egx.PREC_MIXED])
def test_device_krylov_control_matches_host_driver(egx_ctx, small_solve, precision, monkeypatch):
    """The Arnoldi decisions taken on the device (default) and by the host
    driver (EGX_KRYLOV_HOST=1) give the same iteration counts, apply counts
    and solutions (complex128: to 1e-12; the mixed form, whose complex64
    inner vectors can round differently when a coefficient differs in its
    last bit: both to their 1e-6 target, jQ within 2e-6)."""
    from extreme_gb300.forward import ForwardSettings, MixedSettings, Mt3DForwardSolver
    m, om, G, out = small_solve
    solver = Mt3DForwardSolver(ForwardSettings(residual=1e-8, outer_buffer_length=20), precision=precision,
                               mixed=MixedSettings(tol=1e-6), ctx=egx_ctx)
    sols = {}
    for mode in ("0", "1"):
        monkeypatch.setenv("EGX_KRYLOV_HOST", mode)
        sols[mode] = solver.solve(m, 0.1)
    a, b = sols["0"], sols["1"]
    for i in range(2):
        if precision == egx.PREC_FP64:
            assert a.results[i]["iterations"] == b.results[i]["iterations"]
            assert a.results[i]["n_applies"] == b.results[i]["n_applies"]
            assert rel(a.jq[i], b.jq[i]) < 1e-12
        else:
            assert a.results[i]["true_be"] < 1e-6 and b.results[i]["true_be"] < 1e-6
            assert rel(a.jq[i], b.jq[i]) < 2e-6
