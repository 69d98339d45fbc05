"""GPU: Green-tensor reuse across solves (``TensorCache.cs``).

* Two models with the same geometry and background but different anomaly
  conductivities (an inversion step): solving both through one
  ``TensorCache`` builds the anomaly-to-anomaly tensor once and gives the
  same currents as solving each with its own tensor.
* The context's level-tensor cache: a repeated level is a hit with identical
  fields; a changed background, frequency or shift is a build, never a stale
  hit; capacity 0 always builds.
"""
import numpy as np
import pytest

from extreme_gb300.forward import ForwardSettings, Mt3DForwardSolver, TensorCache
from extreme_gb300.model import freq_to_omega, random_model

pytestmark = pytest.mark.gpu


def test_atoa_cache_reused_across_anomalies(egx_ctx):
    m1 = random_model(16, 16, 8, seed=21)
    m2 = random_model(16, 16, 8, seed=21)
    rng = np.random.default_rng(1)
    m2.sigma *= 10.0 ** rng.uniform(-0.5, 0.5, m2.sigma.shape)  # same background, new anomaly
    solver = Mt3DForwardSolver(ForwardSettings(residual=1e-9, outer_buffer_length=20), ctx=egx_ctx)
    cache = TensorCache()
    try:
        a1 = solver.solve(m1, 0.1, tensors=cache)
        a2 = solver.solve(m2, 0.1, tensors=cache)
        assert len(cache) == 1
        solver.solve(m1, 1.0, tensors=cache)
        assert len(cache) == 2
    finally:
        cache.free()
    b1 = solver.solve(m1, 0.1)
    b2 = solver.solve(m2, 0.1)
    np.testing.assert_array_equal(a1.jq, b1.jq)
    np.testing.assert_array_equal(a2.jq, b2.jq)


def test_level_cache_hits_and_keys(egx_ctx):
    m = random_model(12, 10, 6, seed=5)
    n = m.nx * m.ny * 3 * m.nz
    rng = np.random.default_rng(2)
    jq = rng.standard_normal((2, n)) + 1j * rng.standard_normal((2, n))
    om = freq_to_omega(0.3)
    egx_ctx.level_cache(4)
    h0, b0 = egx_ctx.level_cache()
    e1, _ = egx_ctx.level_fields(m, om, jq, z=0.0)
    e2, _ = egx_ctx.level_fields(m, om, jq, z=0.0)
    h1, b1 = egx_ctx.level_cache()
    assert (h1 - h0, b1 - b0) == (1, 1)
    np.testing.assert_array_equal(e1, e2)
    # other frequency, shift, background: builds, and the results are those of a fresh build
    egx_ctx.level_fields(m, freq_to_omega(0.5), jq, z=0.0)
    egx_ctx.level_fields(m, om, jq, z=0.0, shift_x=250.0)
    m_bg = random_model(12, 10, 6, seed=5)
    m_bg.section.sigma = m_bg.section.sigma * 2.0
    e_bg, _ = egx_ctx.level_fields(m_bg, om, jq, z=0.0)
    h2, b2 = egx_ctx.level_cache()
    assert (h2 - h1, b2 - b1) == (0, 3)
    egx_ctx.level_cache(0)
    e_fresh, _ = egx_ctx.level_fields(m_bg, om, jq, z=0.0)
    e_again, _ = egx_ctx.level_fields(m, om, jq, z=0.0)
    h3, b3 = egx_ctx.level_cache()
    assert (h3 - h2, b3 - b2) == (0, 2)
    np.testing.assert_array_equal(e_bg, e_fresh)
    np.testing.assert_array_equal(e_again, e1)
    assert not np.allclose(e_bg, e1)
    egx_ctx.level_cache(4)
