"""GPU: parity on the medium and precision generators (5-layer random
background, depth-growing layers dz_k = 100 m * 1.1^k, 20 random boxes,
500 m cells), not only on the small three-layer model.

Medium generator at 32x32x32 (full oracle pipeline):
* the FP64 Green tensor built on the device within 1e-10 of the oracle's at
  1e-3 and 10 Hz (the ends of the configuration's frequency range);
* the complex128 operator apply (A and chi0) on the device-built tensor
  within 1e-10 of the oracle's apply (``ConvolutionOperator.cs:45-327``);
* at 1e-3 Hz the complex128 FGMRES solve of both polarisations
  (FGMRES(20)+GMRES(10), tol 1e-8): iteration counts equal to the oracle's,
  jQ, the surface E and H and the off-diagonal apparent resistivity and
  phase within 10x the tolerance of the oracle's
  (``Mt3DForwardSolver.cs:297-337``, ``ResponseFunctionsCalculator.cs:36-51``);
* the mixed-precision solve (tol 1e-6) within 1e-5 of the complex128 one
  for the same quantities.

Precision generator at 48x48x48 (nz = 48: the complex64 sub-block
contraction of the precision configuration):
* the complex128 apply within 1e-10 and the complex64 two-source apply
  within 2e-5 of the oracle's apply on the downloaded device-built tensor;
* at four frequencies 1e-3..10 Hz, the mixed solve's jQ, surface E and H
  and off-diagonal rho_a / phase within 1e-5 of a complex128 solve to 1e-9.

Medium configuration at its full size, 128x128x32: the complex128 apply
within 1e-10 of the oracle's apply on the downloaded device-built tensor.
"""
import numpy as np
import pytest

from extreme_gb300 import egx
from extreme_gb300.forward import ForwardSettings, MixedSettings, Mt3DForwardSolver
from extreme_gb300.model import OmegaModel, freq_to_omega, medium_model, scaled_model
from oracle import atoo, green, mt
from oracle import operator as op

pytestmark = pytest.mark.gpu
COMPS = ("xx", "xy", "yy", "zz", "xz", "yz")


def rel(a, b):
    return np.linalg.norm(np.ravel(a) - np.ravel(b)) / np.linalg.norm(np.ravel(b))


def offdiag(a):
    """xy and yx entries of [sites, 2, 2] responses."""
    a = np.asarray(a).reshape(-1, 2, 2)
    return np.stack([a[:, 0, 1], a[:, 1, 0]])


def _apply_pair(ctx, G, om, m, rng, tol=1e-10, chunk=None):
    """Device apply (A and chi0) against the oracle's on the same tensor."""
    n = m.nx * m.ny * 3 * m.nz
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    g = ctx.green_upload(G, m.nx, m.ny, m.nz)
    try:
        for t in (op.OP_A, op.OP_CHI0):
            ctx.op_prepare(g, om.zeta, om.zeta0, m.layer_thickness, t)
            y = ctx.op_apply(x)
            want = op.apply(G, om, x, t, chunk=chunk)
            assert rel(y, want) < tol, (t, rel(y, want))
    finally:
        g.free()


# ---------------------------------------------------------------- medium generator, 32x32x32

MEDIUM_SMALL = (32, 32, 32, 5)


@pytest.fixture(scope="module")
def medium_small():
    m = scaled_model(*MEDIUM_SMALL[:3], seed=MEDIUM_SMALL[3])
    return m


@pytest.mark.parametrize("f", [1e-3, 10.0])
def test_medium_generator_green_and_apply(egx_ctx, medium_small, f):
    m = medium_small
    om = OmegaModel.build(m, f)
    want = green.green_tensor(om, 10)
    g = egx_ctx.green_build(m, om.omega, 10, egx.PREC_FP64)
    try:
        got = g.download()
    finally:
        g.free()
    for c in COMPS:
        assert rel(got[c], want[c]) < 1e-10, (c, rel(got[c], want[c]))
    _apply_pair(egx_ctx, got, om, m, np.random.default_rng(int(f * 1000) + 1))


@pytest.fixture(scope="module")
def medium_solves(egx_ctx, medium_small):
    """Oracle and device solves at 1e-3 Hz with the surface responses."""
    m = medium_small
    f = 1e-3
    om = OmegaModel.build(m, f)
    G = green.green_tensor(om, 10)
    outs = {p: mt.solve_polarization(om, G, p, m_out=20, m_in=10, tol=1e-8) for p in "xy"}
    want = atoo.level_responses(om, atoo.Level(0.0, 0.0, 0.0), outs["x"].jq, outs["y"].jq)
    plain = Mt3DForwardSolver(ForwardSettings(residual=1e-8, outer_buffer_length=20), ctx=egx_ctx)
    sol64 = plain.solve(m, f, levels=[0.0])
    mixed = Mt3DForwardSolver(ForwardSettings(), precision=egx.PREC_MIXED, mixed=MixedSettings(tol=1e-6),
                              ctx=egx_ctx)
    sol32 = mixed.solve(m, f, levels=[0.0])
    return m, outs, want, sol64, sol32


def test_medium_generator_fp64_solve_matches_oracle(medium_solves):
    m, outs, want, sol, _ = medium_solves
    tol = 10 * 1e-8
    lv = sol.levels[0]
    for i, p in enumerate("xy"):
        assert sol.results[i]["converged"]
        assert sol.results[i]["iterations"] == outs[p].result.iterations
        assert rel(sol.jq[i], outs[p].jq) < tol
        assert rel(lv.e[i], want["e%d" % i]) < tol
        assert rel(lv.h[i], want["h%d" % i]) < tol
    assert rel(offdiag(lv.rho), offdiag(want["rho"])) < tol
    assert rel(offdiag(lv.phase), offdiag(want["phase"])) < tol


def test_medium_generator_mixed_solve_matches_fp64(medium_solves):
    m, _, _, s64, s32 = medium_solves
    a, b = s32.levels[0], s64.levels[0]
    for i in range(2):
        assert s32.results[i]["converged"] and s32.results[i]["true_be"] < 1e-6
        assert rel(s32.jq[i], s64.jq[i]) < 1e-5
        assert rel(a.e[i], b.e[i]) < 1e-5
        assert rel(a.h[i], b.h[i]) < 1e-5
    assert rel(offdiag(a.rho), offdiag(b.rho)) < 1e-5
    assert rel(offdiag(a.phase), offdiag(b.phase)) < 1e-5


# ---------------------------------------------------------------- precision generator, 48x48x48

@pytest.fixture(scope="module")
def precision_small():
    return scaled_model(48, 48, 48, seed=7)


def test_precision_generator_applies_match_oracle(egx_ctx, precision_small):
    m = precision_small
    f = m.frequencies[1]
    om = OmegaModel.build(m, f)
    g = egx_ctx.green_build(m, om.omega, 10, egx.PREC_MIXED)
    try:
        G = g.download()
        n = m.nx * m.ny * 3 * m.nz
        rng = np.random.default_rng(8)
        egx_ctx.op_prepare(g, om.zeta, om.zeta0, m.layer_thickness, op.OP_A)
        x2 = (rng.standard_normal((2, n)) + 1j * rng.standard_normal((2, n))).astype(np.complex64)
        y2 = egx_ctx.op_apply_c64(x2.reshape(-1), nrhs=2).reshape(2, n)
        for i in range(2):
            want = op.apply(G, om, x2[i].astype(np.complex128), op.OP_A)
            assert rel(y2[i], want) < 2e-5, (i, rel(y2[i], want))
    finally:
        g.free()
    _apply_pair(egx_ctx, G, om, m, np.random.default_rng(9))


def test_precision_generator_mixed_fields_within_1e5(egx_ctx, precision_small):
    m = precision_small
    plain = Mt3DForwardSolver(ForwardSettings(residual=1e-9, outer_buffer_length=20), ctx=egx_ctx)
    mixed = Mt3DForwardSolver(ForwardSettings(), precision=egx.PREC_MIXED, mixed=MixedSettings(tol=1e-6),
                              ctx=egx_ctx)
    for f in m.frequencies:
        s64 = plain.solve(m, f, levels=[0.0])
        s32 = mixed.solve(m, f, levels=[0.0])
        a, b = s32.levels[0], s64.levels[0]
        errs = {"jq": max(rel(s32.jq[i], s64.jq[i]) for i in range(2)),
                "e": max(rel(a.e[i], b.e[i]) for i in range(2)),
                "h": max(rel(a.h[i], b.h[i]) for i in range(2)),
                "rho": rel(offdiag(a.rho), offdiag(b.rho)),
                "phase": rel(offdiag(a.phase), offdiag(b.phase))}
        assert all(r["converged"] and r["true_be"] < 1e-6 for r in s32.results), (f, s32.results)
        assert max(errs.values()) < 1e-5, (f, errs)


# ---------------------------------------------------------------- medium configuration, full size

def test_medium_full_size_apply_matches_oracle(egx_ctx):
    m = medium_model(seed=1)
    f = m.frequencies[2]
    om = OmegaModel.build(m, f)
    g = egx_ctx.green_build(m, freq_to_omega(f), 10, egx.PREC_FP64)
    try:
        G = g.download()
    finally:
        g.free()
    _apply_pair(egx_ctx, G, om, m, np.random.default_rng(10), chunk=16)
