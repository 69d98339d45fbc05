"""Oracle (TEST INFRASTRUCTURE ONLY, see ``oracle/__init__.py``): the MT source field and the CIE pipeline around the solve.

* 1-D plane-wave field at lambda = 0 (``Extreme.Cartesian.Magnetotellurics/PlaneWaveCalculator.cs:11-83``
  with the single-lambda recursions of ``Green/Scalar/Impl/PlanCalculator.cs:173-314``);
* normal field on the anomaly layers, thickness-averaged, in the x (pol X)
  or y (pol Y) component (``Solver/Mt3DForwardSolver.cs:251-275``);
* ``jS = (zeta - zeta0) E0``, ``chi0 = K_chi0 jS``, solve ``A chi = chi0``
  with ``x0 = chi0``, ``Es = (2 sqrt(Re zeta0) chi - jS)/(zeta + conj zeta0)``,
  ``jQ = Es (zeta - zeta0) + jS`` (``Forward/ForwardSolver.cs:186-436``,
  ``Forward/ForwardSolverGenerics.cs:30-50``).
"""
import numpy as np

from . import fgmres as _fg
from . import operator as _op
from .green import corresponding_layer

MU0 = 4.0 * np.pi * 1.0e-7


def _plane_wave_container(om, rc_depth):
    """``PlaneWaveCalculator.PrepareContainer`` at lambda = 0."""
    m = om.model
    tops = m.section.layer_tops()
    thick = m.section.thickness
    zb = om.zeta_bg
    L = len(zb)
    i_omega = complex(0.0, om.omega)
    eta = np.array([np.sqrt(0.0 - i_omega * zb[k] * MU0) for k in range(L)])
    ex = np.array([np.exp(-2 * eta[k] * thick[k]) for k in range(L)])
    q = np.zeros(L, np.complex128)
    n = L - 1
    part = 1.0 * (eta[n] / eta[n - 1])
    q[n - 1] = (1 - part) / (1 + part)
    for k in range(n - 1, 1, -1):
        qexp = q[k] * ex[k]
        part = 1.0 * (eta[k] / eta[k - 1]) * ((qexp - 1) / (qexp + 1))
        q[k - 1] = (1 + part) / (1 - part)
    p = np.zeros(L, np.complex128)
    p[1] = (eta[1] - eta[0]) / (eta[1] + eta[0])
    for k in range(1, L - 1):
        pexp = p[k] * ex[k]
        part = 1.0 * (eta[k] / eta[k + 1]) * ((pexp - 1) / (pexp + 1))
        p[k + 1] = (1 + part) / (1 - part)
    tr = corresponding_layer(tops, thick, 0.0)
    rc = corresponding_layer(tops, thick, rc_depth)
    s, r = max(rc, tr), min(rc, tr)
    A = np.zeros((L, L), np.complex128)
    for nn in range(s, r - 1, -1):
        prev = 1.0 / (eta[nn] * (1 - p[nn] * q[nn] * ex[nn]))
        A[nn, nn] = prev
        for k in range(nn - 1, r - 1, -1):
            f = ((1 + p[k + 1]) / (1 + p[k] * ex[k])) * np.exp((eta[k + 1] - eta[k]) * tops[k + 1])
            prev = f * prev
            A[k, nn] = prev
            A[nn, k] = prev
    return tops, q, A, rc, tr


def plane_wave_e(om, depth, thick=0.0):
    """``PlaneWaveCalculator.CalculateFieldE`` (``PlaneWaveCalculator.cs:11-40``)."""
    tops, q, A, rc, tr = _plane_wave_container(om, depth)
    zb = om.zeta_bg
    kkr = 1j * om.omega * MU0 * zb[rc]
    ikr = 1j * np.sqrt(kkr)
    kk1 = 1j * om.omega * MU0 * zb[tr]
    ik1 = 1j * np.sqrt(kk1)
    dr1 = tops[rc + 1]
    d2 = tops[tr + 1]
    zr = depth
    a = A[rc, tr] / A[tr, tr]
    if thick == 0:
        upper = np.exp(ikr * zr) + q[rc] * np.exp(ikr * (2 * dr1 - zr))
    else:
        z1 = zr - thick / 2
        z2 = zr + thick / 2
        u1 = np.exp(ikr * z1) - q[rc] * np.exp(ikr * (2 * dr1 - z1))
        u2 = np.exp(ikr * z2) - q[rc] * np.exp(ikr * (2 * dr1 - z2))
        upper = (u2 - u1) / (z2 - z1) / ikr
    lower = 1 + q[tr] * np.exp(ik1 * (2 * d2))
    return a * (upper / lower)


def plane_wave_h(om, depth):
    """``PlaneWaveCalculator.CalculateFieldH`` (``PlaneWaveCalculator.cs:42-64``)."""
    tops, q, A, rc, tr = _plane_wave_container(om, depth)
    zb = om.zeta_bg
    kkr = 1j * om.omega * MU0 * zb[rc]
    ikr = 1j * np.sqrt(kkr)
    kk1 = 1j * om.omega * MU0 * zb[tr]
    ik1 = 1j * np.sqrt(kk1)
    dr1 = tops[rc + 1]
    d2 = tops[tr + 1]
    a = A[rc, tr] / A[tr, tr]
    upper = np.exp(ikr * depth) - q[rc] * np.exp(ikr * (2 * dr1 - depth))
    lower = 1 + q[tr] * np.exp(ik1 * (2 * d2))
    return (np.sqrt(kkr) / (om.omega * MU0)) * a * (upper / lower)


def normal_field(om, pol):
    """E0 on the anomaly (``Mt3DForwardSolver.CalculateNormalFieldFromSource``)."""
    m = om.model
    e = np.zeros((m.nx, m.ny, 3, m.nz), np.complex128)
    c = 0 if pol == "x" else 1
    for k in range(m.nz):
        mid = m.layer_depth[k] + m.layer_thickness[k] / 2
        e[:, :, c, k] = plane_wave_e(om, mid, m.layer_thickness[k])
    return e.reshape(-1)


def scattered_current(om, e0):
    m = om.model
    d = (om.zeta - om.zeta0[None, None, :])[:, :, None, :]
    return (d * e0.reshape(m.nx, m.ny, 3, m.nz)).reshape(-1)


def e_scattered(om, chi, js):
    m = om.model
    z0 = om.zeta0
    sq = np.sqrt(z0.real).astype(np.complex128)[None, None, None, :]
    den = (om.zeta + np.conj(z0)[None, None, :])[:, :, None, :]
    c = chi.reshape(m.nx, m.ny, 3, m.nz)
    j = js.reshape(m.nx, m.ny, 3, m.nz)
    return ((2 * sq * c - j) / den).reshape(-1)


def j_q(om, es, js):
    m = om.model
    d = (om.zeta - om.zeta0[None, None, :])[:, :, None, :]
    return (es.reshape(m.nx, m.ny, 3, m.nz) * d + js.reshape(m.nx, m.ny, 3, m.nz)).reshape(-1)


class SolveOutput:
    pass


def solve_polarization(om, G, pol, m_out=20, m_in=10, tol=1e-8, max_restarts=100, make_op=None):
    """One source: ``SolveForOneSource`` up to ``jQ``. ``make_op(G, om,
    type)`` builds the prepared operators (default
    :class:`oracle.operator.Operator`; the CPU baseline passes the threaded
    one of ``oracle/cpu_apply.py``)."""
    make_op = make_op or _op.Operator
    e0 = normal_field(om, pol)
    js = scattered_current(om, e0)
    chi0 = make_op(G, om, _op.OP_CHI0)(js)
    A = make_op(G, om, _op.OP_A)
    solver = _fg.fgmres_with_gmres(A, m_out, m_in, tol, max_restarts)
    chi, res = solver.solve(chi0, chi0.copy())
    es = e_scattered(om, chi, js)
    out = SolveOutput()
    out.e0, out.js, out.chi0, out.chi, out.es = e0, js, chi0, chi, es
    out.jq = j_q(om, es, js)
    out.result = res
    out.n_applies = A.n_applies + 1
    return out
