"""CPU: the oracle's observation-level path.

* The volume-to-point scalars (receiver at a point) are the thin-layer limit
  of the volume-to-volume scalars, which are pinned to the reference's own C
  (``test_oracle.py``): ``I_vtv(receiver [z-e, z+e]) / 2e -> I_vtp(z)``.
* The level plan adds the zero radius exactly when a knot can sit on the
  axis (``ScalarPlansCreater.cs:51-66,240-262``).
* ``egx_mt_responses`` (host arithmetic in the C library, no GPU work)
  equals the oracle's impedance, apparent resistivity and phase, and a
  homogeneous half-space gives rho_a = rho and phase = 45 degrees.
"""
import warnings

import numpy as np
import pytest

from extreme_gb300.model import CartesianModel, OmegaModel, Section1D, small_model
from oracle import atoo, green


def rel(a, b):
    return np.linalg.norm(np.ravel(a) - np.ravel(b)) / np.linalg.norm(np.ravel(b))


@pytest.mark.parametrize("f", [0.1, 10.0])
def test_point_scalars_are_thin_layer_limit_of_volume_scalars(f):
    warnings.simplefilter("ignore", RuntimeWarning)
    m = small_model()
    om = OmegaModel.build(m, f)
    hk = green.Hankel()
    items, _ = atoo.level_plan(m, atoo.Level(0.0), 10, hk)
    rho, lam = items[3]
    k = 3
    z1, z2 = m.layer_depth[k], m.layer_depth[k] + m.layer_thickness[k]
    eps = 0.01
    # receivers above the layer in the same background layer, below it in the next one
    for zr in (1000.0, 1500.0, 2100.0, 2700.0):
        vtp = atoo.vtp_scalars_for_item(om, hk, rho, lam, [(zr, z1, z2)], "E")
        vtv = green.scalars_for_item(om, hk, rho, lam, [(zr - eps, zr + eps, z1, z2)], [1, 2, 3, 4, 5])
        for i in (1, 2, 3, 4, 5):
            dev = np.max(np.abs(vtv[i][0] / (2 * eps) - vtp[i][0])) / np.max(np.abs(vtp[i][0]))
            assert dev < 5e-9, (zr, i, dev)


def test_level_plan_zero_radius():
    m = small_model()
    hk = green.Hankel()
    _, add0 = atoo.level_plan(m, atoo.Level(0.0), 10, hk)
    assert not add0                     # receivers on cell centres: rho >= dx/2
    items, add0 = atoo.level_plan(m, atoo.Level(0.0, m.dx / 2, 0.0), 10, hk)
    assert add0                         # a knot on the axis
    assert items[0][0][0] == pytest.approx(min(m.dx, m.dy) * atoo.RHO_MIN_FORCED_FACTOR)


def test_mt_responses_c_matches_oracle():
    from extreme_gb300 import egx
    rng = np.random.default_rng(3)
    n = 37
    f = [rng.standard_normal((n, 3)) + 1j * rng.standard_normal((n, 3)) for _ in range(4)]
    omega = 2 * np.pi * 0.37
    z, rho, ph = egx.mt_responses(f[0], f[1], f[2], f[3], omega)
    zo = atoo.impedance(f[0], f[1], f[2], f[3])
    ro, po = atoo.rho_phase(zo, omega)
    assert rel(z, zo) < 1e-14
    assert rel(rho, ro) < 1e-14
    np.testing.assert_allclose(ph, po, rtol=0, atol=1e-12)


def test_half_space_responses():
    """Homogeneous earth under air, no anomaly: rho_a = rho, phase 45 deg."""
    sigma = 0.01
    section = Section1D(0.0, np.array([0.0, 5000.0, 0.0]), np.array([0.0, sigma, sigma]))
    m = CartesianModel(4, 4, 100.0, 100.0, section, np.array([0.0]), np.array([100.0]),
                       np.full((4, 4, 1), sigma)).validate()
    om = OmegaModel.build(m, 1.0)
    e0, h0 = atoo.normal_fields(om, 0.0, 0)
    e1, h1 = atoo.normal_fields(om, 0.0, 1)
    z = atoo.impedance(e0[None], e1[None], h0[None], h1[None])
    rho, ph = atoo.rho_phase(z, om.omega)
    assert rho[0, 0, 1] == pytest.approx(1 / sigma, rel=1e-6)
    assert rho[0, 1, 0] == pytest.approx(1 / sigma, rel=1e-6)
    assert abs(abs(ph[0, 0, 1]) - 45.0) < 1e-4 and abs(abs(ph[0, 1, 0]) - 135.0) < 1e-4
