"""GPU: failure paths of the solve, made on the host (no device fault).

* Arnoldi breakdown (``||w|| = 0``) and the exact initial guess of
  ``GmresSolver.Solve`` (``Extreme.Fgmres/Gmres.cs:77-143``,
  ``CheckForExactSolution`` ``:104-107,350-356``) through
  ``egx_fgmres_solve``, on the CIE operator of a model without anomaly
  (zeta = zeta0 in every cell: r = 0, so A = I exactly in complex128).
  Iterations, apply counts and results equal the oracle's on the same cases
  (``tests/test_oracle_failure.py``).
* The learned preconditioner's fallback: a NaN written by the host over the
  network's output (``egx_learned_inject_nonfinite``) makes the inner solve
  fail; the GMRES-preconditioned solve redoes it and the mixed solve still
  reaches its 1e-6 true residual.
"""
import os

import numpy as np
import pytest

from extreme_gb300 import egx
from extreme_gb300.model import OmegaModel
from oracle import fgmres

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "tiny.npz")
COMPS = ("xx", "xy", "yy", "zz", "xz", "yz")


@pytest.fixture(scope="module")
def identity_op(egx_ctx):
    from tests.golden.make_golden import tiny_model
    gold = np.load(GOLD)
    m = tiny_model()
    om = OmegaModel.build(m, 1.0)
    G = {c: gold["oracle_G_" + c] for c in COMPS}
    g = egx_ctx.green_upload(G, m.nx, m.ny, m.nz)
    zeta = np.broadcast_to(om.zeta0, om.zeta.shape).copy()
    egx_ctx.op_prepare(g, zeta, om.zeta0, m.layer_thickness, egx.OP_A)
    yield m, m.nx * m.ny * 3 * m.nz
    g.free()


def _oracle(b, x0):
    calls = []

    def apply(v):
        calls.append(1)
        return v.copy()
    x, r = fgmres.fgmres_with_gmres(apply, 5, 3, 1e-9, 10).solve(b, x0.copy())
    return x, r, len(calls)


def test_identity_apply_is_exact(egx_ctx, identity_op):
    _, n = identity_op
    rng = np.random.default_rng(3)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    np.testing.assert_array_equal(egx_ctx.op_apply(x), x)


def test_arnoldi_breakdown(egx_ctx, identity_op):
    _, n = identity_op
    b = np.zeros(n, np.complex128)
    b[5] = 2.0
    x, r = egx_ctx.fgmres_solve(b, np.zeros_like(b), m_out=5, m_in=3, tol=1e-9, max_restarts=10)
    xo, ro, calls = _oracle(b, np.zeros_like(b))
    assert r["converged"] and r["iterations"] == ro.iterations == 1
    assert r["arnoldi_be"] == 0 and r["true_be"] == 0
    assert r["n_applies"] == calls == 4
    np.testing.assert_array_equal(x, b)
    np.testing.assert_array_equal(xo, b)


def test_near_breakdown(egx_ctx, identity_op):
    _, n = identity_op
    rng = np.random.default_rng(4)
    b = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    x, r = egx_ctx.fgmres_solve(b, np.zeros_like(b), m_out=5, m_in=3, tol=1e-9, max_restarts=10)
    xo, ro, _ = _oracle(b, np.zeros_like(b))
    assert r["converged"] and r["iterations"] == ro.iterations == 1
    assert r["true_be"] < 1e-15
    np.testing.assert_allclose(x, b, rtol=1e-14)


def test_exact_initial_guess(egx_ctx, identity_op):
    _, n = identity_op
    rng = np.random.default_rng(5)
    b = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    x, r = egx_ctx.fgmres_solve(b, b, m_out=5, m_in=3, tol=1e-9, max_restarts=10)
    _, ro, calls = _oracle(b, b)
    assert r["converged"] and r["iterations"] == ro.iterations == 1
    assert r["arnoldi_be"] == 0 and r["true_be"] == 0
    assert r["n_applies"] == calls == 1
    np.testing.assert_array_equal(x, b)


def test_zero_rhs(egx_ctx, identity_op):
    _, n = identity_op
    x0 = np.ones(n, np.complex128)
    x, r = egx_ctx.fgmres_solve(np.zeros(n, np.complex128), x0, m_out=5, m_in=3, tol=1e-9, max_restarts=10)
    assert r["converged"] and r["iterations"] == 0 and r["n_applies"] == 0
    np.testing.assert_array_equal(x, x0)


def test_learned_fallback_on_nonfinite_output(egx_ctx):
    """An untrained network (the identity map), its first output poisoned
    with NaN from the host: the inner solve stops at the non-finite norm,
    the fallback runs, the solve converges; disarmed, the next solve uses
    the network again and converges."""
    from extreme_gb300.forward import ForwardSettings, MixedSettings, Mt3DForwardSolver
    from extreme_gb300.learned import log_conductivity
    from extreme_gb300.model import scaled_model
    m = scaled_model(16, 16, 4, seed=5)
    f = 1.0
    net = egx.SpectralNet(egx_ctx, m.nx, m.ny, m.nz, width=8, layers=1, seed=0)
    solver = Mt3DForwardSolver(ForwardSettings(), precision=egx.PREC_MIXED, mixed=MixedSettings(tol=1e-6),
                               ctx=egx_ctx)
    try:
        net.set_model(log_conductivity(m, f))
        egx_ctx.set_learned(net)
        u0, f0 = egx_ctx.learned_stats()
        egx_ctx.learned_inject_nonfinite(1)
        sol = solver.solve(m, f)
        u1, f1 = egx_ctx.learned_stats()
        assert u1 > u0 and f1 - f0 >= 1
        assert all(r["converged"] and r["true_be"] < 1e-6 for r in sol.results), sol.results
        egx_ctx.learned_inject_nonfinite(0)
        sol = solver.solve(m, f)
        u2, f2 = egx_ctx.learned_stats()
        assert u2 > u1
        assert all(r["converged"] and r["true_be"] < 1e-6 for r in sol.results), sol.results
    finally:
        egx_ctx.learned_inject_nonfinite(0)
        egx_ctx.set_learned(None)
        net.free()
