"""GPU: fields at observation levels and the MT responses through the C ABI
against the oracle.

* Anomalous E and H from the device-built level tensors for random currents,
  at levels above, inside and below the anomaly, with and without lateral
  shift (the half-cell shift puts a knot on the axis: zero radius in the
  plan): complex128 throughout, <= 1e-10 relative.
* End to end on the 32x32x8 model: jQ of both polarisations (FGMRES to
  1e-8), level fields at the surface, total fields, apparent resistivity and
  phase within 10x the FGMRES tolerance of the oracle pipeline.
"""
import numpy as np
import pytest

from extreme_gb300 import egx
from extreme_gb300.forward import ForwardSettings, Mt3DForwardSolver
from extreme_gb300.model import OmegaModel, small_model
from oracle import atoo, green, mt

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(np.ravel(a) - np.ravel(b)) / np.linalg.norm(np.ravel(b))


def _tiny():
    from tests.golden.make_golden import tiny_model
    m = tiny_model()
    return m, OmegaModel.build(m, 1.0)


@pytest.mark.parametrize("z, sx, sy", [(0.0, 0.0, 0.0), (0.0, 200.0, 100.0), (400.0, 0.0, 0.0),
                                       (1000.0, 100.0, 0.0)])
def test_level_fields_match_oracle(egx_ctx, z, sx, sy):
    m, om = _tiny()
    rng = np.random.default_rng(int(z) + 7)
    n = m.nx * m.ny * 3 * m.nz
    jq = rng.standard_normal((2, n)) + 1j * rng.standard_normal((2, n))
    e, h = egx_ctx.level_fields(m, om.omega, jq, z=z, shift_x=sx, shift_y=sy)
    lv = atoo.Level(z, sx, sy)
    ge = atoo.level_tensor(om, lv, "E")
    gh = atoo.level_tensor(om, lv, "H")
    for i in range(2):
        assert rel(e[i], atoo.anomaly_field(om, ge, jq[i], "E")) < 1e-10, (i, "E")
        assert rel(h[i], atoo.anomaly_field(om, gh, jq[i], "H")) < 1e-10, (i, "H")


def test_host_out_buffers_page_locked(egx_ctx):
    """Caller-supplied page-locked host outputs: jQ of the solve and the level
    fields written in place, equal to the allocating calls; a wrong dtype or
    size raises before anything runs."""
    import torch
    m, om = _tiny()
    n = m.nx * m.ny * 3 * m.nz
    g = egx_ctx.green_build(m, om.omega, 10)
    try:
        from extreme_gb300.forward import model_zeta
        zeta = model_zeta(m, om.omega)
        e0 = np.stack([egx.normal_field(m, om.omega)] * 2)
        kw = dict(fgmres=dict(m_out=15, m_in=10, tol=1e-8, max_restarts=50))
        jq_a, _, _ = egx_ctx.solve_sources(g, zeta[0], zeta[1], m.layer_thickness, e0, [0, 1], **kw)
        pin_jq = torch.empty((2, n), dtype=torch.complex128, pin_memory=True).numpy()
        jq_b, _, _ = egx_ctx.solve_sources(g, zeta[0], zeta[1], m.layer_thickness, e0, [0, 1], out=pin_jq, **kw)
        assert jq_b.ctypes.data == pin_jq.ctypes.data
        assert rel(pin_jq, jq_a) < 1e-12
        with pytest.raises(ValueError):
            egx_ctx.solve_sources(g, zeta[0], zeta[1], m.layer_thickness, e0, [0, 1],
                                  out=np.empty((2, n), np.complex64), **kw)
    finally:
        g.free()
    e_a, h_a = egx_ctx.level_fields(m, om.omega, jq_a, z=0.0)
    pin = tuple(torch.empty((2, m.nx, m.ny, 3), dtype=torch.complex128, pin_memory=True).numpy() for _ in range(2))
    e_b, h_b = egx_ctx.level_fields(m, om.omega, pin_jq, z=0.0, out=pin)
    assert e_b is pin[0] and h_b is pin[1]
    assert rel(pin[0], e_a) < 1e-12 and rel(pin[1], h_a) < 1e-12
    with pytest.raises(ValueError):
        egx_ctx.level_fields(m, om.omega, jq_a, z=0.0, out=(pin[0][:1], pin[1]))


@pytest.mark.parametrize("shape", [(8, 6, 3), (32, 32, 8)])
def test_mixed_level_tensors_match_fp64(egx_ctx, shape):
    """Level tensors with the complex64 lateral FFT (the mixed form): fields
    within 1e-6 of the FP64 build; the precision is part of the level
    cache's key."""
    from extreme_gb300.model import freq_to_omega, scaled_model
    m = scaled_model(*shape, seed=4)
    omega = freq_to_omega(m.frequencies[1])
    rng = np.random.default_rng(3)
    n = m.nx * m.ny * 3 * m.nz
    jq = rng.standard_normal((2, n)) + 1j * rng.standard_normal((2, n))
    egx_ctx.level_cache(4)
    h0, b0 = egx_ctx.level_cache()
    e64, h64 = egx_ctx.level_fields(m, omega, jq, z=0.0)
    e32, h32 = egx_ctx.level_fields(m, omega, jq, z=0.0, precision=egx.PREC_MIXED)
    e32b, _ = egx_ctx.level_fields(m, omega, jq, z=0.0, precision=egx.PREC_MIXED)
    h1, b1 = egx_ctx.level_cache()
    assert (h1 - h0, b1 - b0) == (1, 2)
    np.testing.assert_array_equal(e32, e32b)
    assert rel(e32, e64) < 1e-6 and rel(h32, h64) < 1e-6, (rel(e32, e64), rel(h32, h64))
    assert rel(e32, e64) > 0   # the complex64 FFT ran


def test_surface_responses_match_oracle(egx_ctx):
    m = small_model()
    f = 0.1
    om = OmegaModel.build(m, f)
    G = green.green_tensor(om, 10)
    outs = {p: mt.solve_polarization(om, G, "xy"[p], m_out=20, m_in=10, tol=1e-8) for p in (0, 1)}
    want = atoo.level_responses(om, atoo.Level(0.0), outs[0].jq, outs[1].jq)

    solver = Mt3DForwardSolver(ForwardSettings(residual=1e-8, outer_buffer_length=20), ctx=egx_ctx)
    sol = solver.solve(m, f)
    e, h = egx_ctx.level_fields(m, om.omega, sol.jq, z=0.0)
    full = {}
    for pol in (0, 1):
        en, hn = atoo.normal_fields(om, 0.0, pol)
        full["e%d" % pol] = e[pol] + en
        full["h%d" % pol] = h[pol] + hn
        assert rel(full["e%d" % pol], want["e%d" % pol]) < 10 * 1e-8
        assert rel(full["h%d" % pol], want["h%d" % pol]) < 10 * 1e-8
    z, rho, ph = egx.mt_responses(full["e0"], full["e1"], full["h0"], full["h1"], om.omega)
    rho_w = want["rho"].reshape(-1, 2, 2)
    ph_w = want["phase"].reshape(-1, 2, 2)
    # off-diagonal rho_a and phase, the quantities MT interprets
    for a, b in ((0, 1), (1, 0)):
        assert rel(rho[:, a, b], rho_w[:, a, b]) < 10 * 1e-8
        assert np.max(np.abs(ph[:, a, b] - ph_w[:, a, b])) < 10 * 1e-8 * 180
    # the same through the solver's observation-level path
    lv = solver.solve(m, f, levels=[0.0]).levels[0]
    assert rel(lv.e[0], want["e0"]) < 10 * 1e-8 and rel(lv.h[1], want["h1"]) < 10 * 1e-8
    for a, b in ((0, 1), (1, 0)):
        assert rel(lv.rho[:, a, b], rho_w[:, a, b]) < 10 * 1e-8


def test_device_responses_match_host(egx_ctx):
    """egx_mt_responses_dev (device fields, the plane wave's normal field
    added per polarisation) gives the host egx_mt_responses of the total
    fields: impedance, apparent resistivity and phase to 1e-12."""
    import torch
    n = 37 * 23
    rng = np.random.default_rng(11)
    e = rng.standard_normal((2, n, 3)) + 1j * rng.standard_normal((2, n, 3))
    h = rng.standard_normal((2, n, 3)) + 1j * rng.standard_normal((2, n, 3))
    en, hn = 0.7 - 0.2j, -1.3 + 0.4j
    omega = 2 * np.pi * 0.3
    dev = torch.device("cuda", 0)
    e_d = torch.from_numpy(e.reshape(-1).view(np.float64).copy()).to(dev)
    h_d = torch.from_numpy(h.reshape(-1).view(np.float64).copy()).to(dev)
    z_d = torch.empty(n * 4 * 2, dtype=torch.float64, device=dev)
    rho_d = torch.empty(n * 4, dtype=torch.float64, device=dev)
    ph_d = torch.empty(n * 4, dtype=torch.float64, device=dev)
    torch.cuda.synchronize(dev)
    egx_ctx.mt_responses_dev(e_d.data_ptr(), h_d.data_ptr(), n, omega, en, hn, z_d.data_ptr(), rho_d.data_ptr(),
                             ph_d.data_ptr())
    et, ht = e.copy(), h.copy()
    et[0, :, 0] += en
    ht[0, :, 1] += hn
    et[1, :, 1] += en
    ht[1, :, 0] -= hn
    z, rho, ph = egx.mt_responses(et[0], et[1], ht[0], ht[1], omega)
    zd = z_d.cpu().numpy().view(np.complex128).reshape(n, 2, 2)
    assert rel(zd, z) < 1e-12
    assert rel(rho_d.cpu().numpy().reshape(n, 2, 2), rho) < 1e-12
    np.testing.assert_allclose(ph_d.cpu().numpy().reshape(n, 2, 2), ph, rtol=0, atol=1e-9)
    with pytest.raises(egx.EgxError):
        egx_ctx.mt_responses_dev(e_d.data_ptr(), h_d.data_ptr(), 0, omega, en, hn, z_d.data_ptr(),
                                 rho_d.data_ptr(), ph_d.data_ptr())
