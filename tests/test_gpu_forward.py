"""GPU: the full forward solve of one frequency (Green tensor on the device,
both polarisations, jQ) through the C ABI against the oracle pipeline.

jQ (the current every observation is computed from) must agree with the
oracle within 10x the FGMRES tolerance; the mixed-precision form within its
1e-6 target residual (checked at 2e-5 relative on the small model).
"""
import numpy as np
import pytest

from extreme_gb300 import egx
from extreme_gb300.forward import ForwardSettings, MixedSettings, Mt3DForwardSolver
from extreme_gb300.model import OmegaModel, small_model
from oracle import green, mt

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(np.ravel(a) - np.ravel(b)) / np.linalg.norm(np.ravel(b))


@pytest.fixture(scope="module")
def oracle_small():
    m = small_model()
    om = OmegaModel.build(m, 0.1)
    G = green.green_tensor(om, 10)
    outs = {p: mt.solve_polarization(om, G, p, m_out=20, m_in=10, tol=1e-8) for p in "xy"}
    return m, om, outs


def test_normal_field_matches_oracle(oracle_small):
    m, om, outs = oracle_small
    e0 = egx.normal_field(m, om.omega)
    want = outs["x"].e0.reshape(m.nx, m.ny, 3, m.nz)[0, 0, 0]
    assert rel(e0, want) < 1e-13
    e, h = egx.plane_wave(m, om.omega, 0.0)
    assert abs(e - mt.plane_wave_e(om, 0.0)) < 1e-13 * abs(e)
    assert abs(h - mt.plane_wave_h(om, 0.0)) < 1e-13 * abs(h)


def test_forward_fp64_matches_oracle(egx_ctx, oracle_small):
    m, om, outs = oracle_small
    solver = Mt3DForwardSolver(ForwardSettings(residual=1e-8, outer_buffer_length=20), ctx=egx_ctx)
    sol = solver.solve(m, 0.1, want_chi=True)
    for i, p in enumerate("xy"):
        assert sol.results[i]["converged"]
        assert sol.results[i]["iterations"] == outs[p].result.iterations
        assert rel(sol.chi[i], outs[p].chi) < 10 * 1e-8
        assert rel(sol.jq[i], outs[p].jq) < 10 * 1e-8


@pytest.mark.parametrize("batch", [True, False])
def test_forward_mixed_matches_oracle(egx_ctx, oracle_small, batch):
    m, om, outs = oracle_small
    solver = Mt3DForwardSolver(ForwardSettings(residual=1e-8), precision=egx.PREC_MIXED,
                               mixed=MixedSettings(tol=1e-6, inner_tol=1e-4, batch=batch), ctx=egx_ctx)
    sol = solver.solve(m, 0.1)
    for i, p in enumerate("xy"):
        assert sol.results[i]["converged"] and sol.results[i]["true_be"] < 1e-6
        assert rel(sol.jq[i], outs[p].jq) < 2e-5
    if batch:   # one stacked solve: shared iteration count
        assert sol.results[0]["iterations"] == sol.results[1]["iterations"]


def test_stacked_sources_scaled_and_zero(egx_ctx, oracle_small):
    """Stacked mixed solve of sources whose right-hand sides differ by 1e6 in
    norm, plus a zero source: every source reaches the tolerance on its own
    residual, the zero source gives jQ = 0, and the scaled source gives the
    scaled currents (the CIE is linear in E0)."""
    m, om, outs = oracle_small
    from extreme_gb300.forward import model_zeta
    zeta, zeta0 = model_zeta(m, om.omega)
    e0 = egx.normal_field(m, om.omega)
    g = egx_ctx.green_build(m, om.omega, 10, egx.PREC_MIXED)
    try:
        e0s = np.stack([e0, 1e6 * e0, np.zeros_like(e0)])
        jq, _, res = egx_ctx.solve_sources(g, zeta, zeta0, m.layer_thickness, e0s, [0, 1, 0],
                                           precision=egx.PREC_MIXED,
                                           mixed=dict(tol=1e-6, inner_tol=1e-4, batch=True))
    finally:
        g.free()
    for r in res:
        assert r["converged"] and r["true_be"] < 1e-6
    assert rel(jq[0], outs["x"].jq) < 2e-5
    assert rel(jq[1] / 1e6, outs["y"].jq) < 2e-5
    assert not np.any(jq[2])


def test_profile_counts_kernels(egx_ctx, oracle_small):
    m, om, outs = oracle_small
    egx_ctx.profile(True)
    solver = Mt3DForwardSolver(ForwardSettings(residual=1e-8, outer_buffer_length=20), ctx=egx_ctx)
    sol = solver.solve(m, 0.1)
    n, ms = egx_ctx.profile_read(egx.K_CONTRACT)
    assert n == sol.results[0]["n_applies"] + sol.results[1]["n_applies"] - 1  # chi0 applies share one launch
    assert ms > 0
    egx_ctx.profile(False)


def test_dot_products_match_numpy(egx_ctx):
    rng = np.random.default_rng(0)
    V = rng.standard_normal((5000, 7)) + 1j * rng.standard_normal((5000, 7))
    w = rng.standard_normal(5000) + 1j * rng.standard_normal(5000)
    got = egx_ctx.dot_products(V, w)
    np.testing.assert_allclose(got, V.conj().T @ w, rtol=1e-12)
