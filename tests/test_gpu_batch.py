"""GPU: the batching form -- many independent solves of uneven meshes run
concurrently on several streams (one context and host thread each), with
the tuner's kernel variants and CUDA-graph inner cycles, give the results of
solving them one by one (to the solver's tolerance), and the tuner returns a
time for every candidate; the graph-captured inner cycle gives bitwise the
launched cycle's results; every apply variant gives the same apply."""
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
        assert set(times) == {(1, False), (3, False), (1, True), (3, True)} and batch.streams in (1, 3)
        assert set(batch.variants) == {(20, 15, 8), (24, 18, 6)}
        got = batch.solve(jobs, levels=[0.0], streams=3)
    finally:
        batch.close()
    # the tuned kernel variants round differently from the built-in ones:
    # both solutions meet the 1e-6 residual, and agree to its order
    one = Mt3DForwardSolver(settings, precision=egx.PREC_MIXED, mixed=mixed, ctx=egx_ctx)
    for (m, f), sol in zip(jobs, got):
        want = one.solve(m, f, levels=[0.0])
        assert all(r["converged"] and r["true_be"] < 1e-6 for r in sol.results)
        assert np.linalg.norm(sol.jq - want.jq) / np.linalg.norm(want.jq) < 2e-6
        rho, rw = sol.levels[0].rho, want.levels[0].rho
        assert np.linalg.norm(rho - rw) / np.linalg.norm(rw) < 1e-5


def test_graph_captured_inner_cycle_matches_launches(egx_ctx):
    """With egx_set_graphs the inner GMRES cycle runs as one replayed CUDA
    graph: the same kernels in the same order, so the same iterations,
    apply counts and (bitwise) currents as the launched cycle, in both
    precisions; the graph was replayed."""
    m = random_model(24, 20, 8, seed=5)
    out = {}
    for graphs in (False, True):
        egx_ctx.set_graphs(graphs)
        r0, _ = egx_ctx.graph_stats()
        for prec in (egx.PREC_FP64, egx.PREC_MIXED):
            solver = Mt3DForwardSolver(ForwardSettings(residual=1e-8), precision=prec,
                                       mixed=MixedSettings(tol=1e-6, inner_tol=1e-4), ctx=egx_ctx)
            out[graphs, prec] = solver.solve(m, 0.3)
        r1, nodes = egx_ctx.graph_stats()
        if graphs:
            assert r1 > r0 and nodes > 0
    egx_ctx.set_graphs(False)
    for prec in (egx.PREC_FP64, egx.PREC_MIXED):
        a, b = out[False, prec], out[True, prec]
        for i in range(2):
            assert a.results[i]["converged"] and b.results[i]["converged"]
            assert a.results[i]["iterations"] == b.results[i]["iterations"]
            assert a.results[i]["n_applies"] == b.results[i]["n_applies"]
        np.testing.assert_array_equal(a.jq, b.jq)


def test_apply_tuner_variants_agree(egx_ctx):
    """Every kernel variant the apply tuner times gives the same apply (to
    complex64 rounding), on the packed Green layout (nz = 7: tensor-core,
    TMA-staged and generic contraction kernels) and the sub-block layout
    (nz = 16, 48: k_contract_sb3 with either reduction layout)."""
    from extreme_gb300.forward import model_zeta
    from extreme_gb300.model import freq_to_omega
    for nz in (7, 16, 48):
        m = random_model(16, 12, nz, seed=6)
        omega = freq_to_omega(1.0)
        g = egx_ctx.green_build(m, omega, 10, egx.PREC_MIXED)
        try:
            zeta, zeta0 = model_zeta(m, omega)
            egx_ctx.op_prepare(g, zeta, zeta0, m.layer_thickness, egx.OP_A)
            tile, var, table = egx_ctx.tune_apply(nrhs=2, reps=2)
            assert (tile, var) in table and len(table) == 9
            n = m.nx * m.ny * 3 * m.nz
            rng = np.random.default_rng(7)
            x = (rng.standard_normal(2 * n) + 1j * rng.standard_normal(2 * n)).astype(np.complex64)
            ys = {}
            for (t, v) in table:
                egx_ctx.apply_variant(t, v)
                ys[t, v] = egx_ctx.op_apply_c64(x, nrhs=2)
            ref = ys[0, 0]
            for k, y in ys.items():
                assert np.linalg.norm(y - ref) / np.linalg.norm(ref) < 1e-5, k
        finally:
            egx_ctx.apply_variant(0, 0)
            g.free()
