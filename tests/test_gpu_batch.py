"""GPU: the batching form -- many independent solves of uneven meshes run
concurrently on several streams (one context and host thread each) give the
results of solving them one by one, and the stream-count tuner returns a
time for every candidate."""
import numpy as np
import pytest

from extreme_gb300 import egx
from extreme_gb300.batch import BatchForwardSolver, is_7smooth, smooth_size
from extreme_gb300.forward import ForwardSettings, MixedSettings, Mt3DForwardSolver
from extreme_gb300.model import random_model

pytestmark = pytest.mark.gpu


def test_smooth_sizes():
    for n in range(32, 200):
        s = smooth_size(n)
        assert is_7smooth(2 * s) and abs(s - n) <= 5


def test_batch_matches_one_by_one(egx_ctx):
    models = [random_model(20, 15, 8, seed=3), random_model(24, 18, 6, seed=4)]
    jobs = [(m, f) for m in models for f in (0.01, 0.3, 5.0)]
    mixed = MixedSettings(tol=1e-6, inner_tol=1e-4)
    settings = ForwardSettings(residual=1e-8)
    batch = BatchForwardSolver(settings, precision=egx.PREC_MIXED, mixed=mixed, streams=3)
    try:
        times = batch.tune(jobs, candidates=(1, 3), sample=3)
        assert set(times) == {1, 3} and batch.streams in (1, 3)
        got = batch.solve(jobs, levels=[0.0], streams=3)
    finally:
        batch.close()
    one = Mt3DForwardSolver(settings, precision=egx.PREC_MIXED, mixed=mixed, ctx=egx_ctx)
    for (m, f), sol in zip(jobs, got):
        want = one.solve(m, f, levels=[0.0])
        assert all(r["converged"] and r["true_be"] < 1e-6 for r in sol.results)
        np.testing.assert_allclose(sol.jq, want.jq, rtol=0, atol=1e-12 * np.abs(want.jq).max())
        np.testing.assert_allclose(sol.levels[0].rho, want.levels[0].rho, rtol=1e-10)
