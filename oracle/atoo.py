"""Oracle: fields at an observation level and the MT responses.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).

Restates, in numpy complex128, the anomaly-to-observation-level path of the
reference after the CIE solve:

* radius plan of a level (``Green/Scalar/ScalarPlansCreater.cs:51-66,110-140,180-262``)
  with the zero radius when a knot can sit on the axis (``GreenScalarCalculator.cs:147-157``,
  ``ScalarMathUtils.cs:33-87``);
* volume-to-point scalars for E and H (``Green/Scalar/Impl/PlanCalculator.cs:60-140,171-315``,
  ``VolumeToPointCalculatorU.cs:21-352``, ``ScalarMathUtils.cs:126-263``);
* the level tensor over the whole (2Nx-1) x (2Ny-1) offset grid, shifted by the
  level's shift (``AtoOLevelGreenTensorCalculator.cs:21-126``,
  ``GreenTensorCalculator.cs:166-552``, ``QSign.cs:31-39``) and its 2-D FFT
  (``AtoOCalculator.cs:166-176``);
* the convolution with jQ (``ToOCalculator.cs:21-125``; ``ZgemvAtoO``,
  ``Native/Native.Matrix/full_zgemv.c:22-26``), normal fields at the level
  (``Mt3DForwardSolver.cs:300-337``) and the impedance, apparent resistivity
  and phase (``ResponseFunctionsCalculator.cs:36-51``, ``PlainTextExporter.cs:322-420``).
"""
import numpy as np

from . import mt as _mt
from .green import (MU0, Hankel, combine, corresponding_layer, integrate, knot, lambdas_for, layer_eta_exp,
                    propagator_chain, reflections, rho_from_max, rho_from_min, segments)

RHO_MIN_FORCED_FACTOR = 0.001
E_COMPS = ("xx", "yy", "zz", "xy", "xz", "yz", "zx", "zy")
H_COMPS = ("xx", "yx", "xy", "xz", "yz", "zx", "zy")


class Level:
    """``ObservationLevel`` (``Extreme.Core/Model/ObservationLevel.cs:4-24``)."""

    def __init__(self, z, shift_x=0.0, shift_y=0.0):
        self.z = float(z)
        self.shift_x = float(shift_x)
        self.shift_y = float(shift_y)


# ------------------------------------------------------------------ plan

def _rho_min_1d(n, cell, shift, anomaly_shift=0.0):
    """``FindRhoMin(numberOfCells, cellSize, shift, anomalyShift)``
    (``ScalarPlansCreater.cs:240-262``); lengths are C# decimal there, exact
    for the centimetre values used here."""
    a_start = anomaly_shift - cell / 2
    a_end = anomaly_shift + cell * n - cell / 2
    y_start = shift - cell / 2
    y_end = y_start + cell * n

    def between(v, lo, hi):
        return lo <= v <= hi
    if between(y_start, a_start, a_end) or between(y_end, a_start, a_end):
        rem = np.fmod(abs(a_start - y_start), cell)
        if rem == 0:
            return cell / 2
        return abs(cell / 2 - rem)
    lc = anomaly_shift
    rc = anomaly_shift + cell * (n - 1)
    return min(min(abs(y_start - lc), abs(y_start - rc)), min(abs(y_end - lc), abs(y_end - rc)))


def _rho_max_four(m, sx, sy, x0, y0):
    """``FindRhoMaxByFourPoints`` (``ScalarPlansCreater.cs:220-233``)."""
    x1 = sx - m.dx / 2
    y1 = sy - m.dy / 2
    x2 = x1 + m.dx * m.nx
    y2 = y1 + m.dy * m.ny
    return max(np.sqrt((x1 - x0) ** 2 + (y1 - y0) ** 2), np.sqrt((x2 - x0) ** 2 + (y1 - y0) ** 2),
               np.sqrt((x2 - x0) ** 2 + (y2 - y0) ** 2), np.sqrt((x1 - x0) ** 2 + (y2 - y0) ** 2))


def level_plan(m, level, n_hankels, hankel):
    """``CreateForAnomalyToObservationLevels`` for one level: list of
    (rho, lambdas) plan items and whether the zero radius is added."""
    rho_min = min(_rho_min_1d(m.nx, m.dx, level.shift_x), _rho_min_1d(m.ny, m.dy, level.shift_y))
    ex, ey = m.dx * (m.nx - 1), m.dy * (m.ny - 1)
    sx, sy = level.shift_x, level.shift_y
    rho_max = max(_rho_max_four(m, sx, sy, 0, 0), _rho_max_four(m, sx, sy, 0, ey),
                  _rho_max_four(m, sx, sy, ex, ey), _rho_max_four(m, sx, sy, ex, 0))
    add_zero = rho_min <= 0
    if add_zero:
        rho_min = min(m.dx, m.dy) * RHO_MIN_FORCED_FACTOR
    step = hankel.rho_step()
    n = abs(n_hankels)
    rho1 = rho_from_min(rho_min, rho_max, step)
    r2, r1 = rho1[-1], rho1[-2]
    lin = (r2 - r1) / n
    items = [rho1]
    for i in range(1, n):
        items.append(rho_from_max(rho_min, r2 - i * lin, step))
    return [(rho, lambdas_for(hankel, rho)) for rho in items], add_zero


# ------------------------------------------------------------------ volume-to-point scalars

def _vtp_terms(eta, tops, zw, z1, z2, r, s):
    """``CalculateT/R/CTop/CBot/DTop/DBot`` of ``VolumeToPointCalculatorU``
    (``VolumeToPointCalculatorU.cs:193-257``) as functions of (a, b, r, s)."""
    def T(a, b, rr, ss):
        t = min(rr, ss)
        dt = tops[t]
        return (np.exp(-eta[rr] * zw - eta[ss] * a + 2 * eta[t] * dt)
                - np.exp(-eta[rr] * zw - eta[ss] * b + 2 * eta[t] * dt))

    def R(a, b, rr, ss):
        bb = max(rr, ss)
        db1 = tops[bb + 1]
        return (np.exp(-2 * eta[bb] * db1 + eta[ss] * b + eta[rr] * zw)
                - np.exp(-2 * eta[bb] * db1 + eta[ss] * a + eta[rr] * zw))

    def ctop(a, b, rr, ss):
        return np.exp(-eta[ss] * a + eta[rr] * zw) - np.exp(-eta[ss] * b + eta[rr] * zw)

    def cbot(a, b, rr, ss):
        return np.exp(-eta[rr] * zw + eta[ss] * b) - np.exp(-eta[rr] * zw + eta[ss] * a)

    def _d(rr, ss):
        t, bb = min(rr, ss), max(rr, ss)
        return -2 * (eta[bb] * tops[bb + 1] - eta[t] * tops[t])

    def dtop(a, b, rr, ss):
        f = _d(rr, ss)
        return np.exp(f + eta[ss] * b - eta[rr] * zw) - np.exp(f + eta[ss] * a - eta[rr] * zw)

    def dbot(a, b, rr, ss):
        f = _d(rr, ss)
        return np.exp(f - eta[ss] * a + eta[rr] * zw) - np.exp(f - eta[ss] * b + eta[rr] * zw)
    return T, R, ctop, cbot, dtop, dbot


def _vtp_u(om, eta, ex, p, q, a_rs, zw, z1, z2, r, s, which, lam):
    """One of ``CalculateU1..U5`` of ``VolumeToPointCalculatorU``
    (``VolumeToPointCalculatorU.cs:21-190,259-345``) for the P/Q/A of the
    current mode."""
    m = om.model
    tops = m.section.layer_tops()
    t, b = min(r, s), max(r, s)
    T, R, ctop, cbot, dtop, dbot = _vtp_terms(eta, tops, zw, z1, z2, r, s)
    if z1 < zw < z2:
        case = "match"
    elif zw >= z2:
        case = "below"
    else:
        case = "above"

    def psi15():
        if case == "match":
            n = r
            return (ctop(zw, z2, n, n) + cbot(z1, zw, n, n)
                    + p[n] * q[n] * (dtop(zw, z2, n, n) + dbot(z1, zw, n, n)))
        if case == "below":
            return cbot(z1, z2, r, s) + p[t] * q[b] * dbot(z1, z2, r, s)
        return ctop(z1, z2, r, s) + p[t] * q[b] * dtop(z1, z2, r, s)

    def psi34():
        if case == "match":
            n = r
            return (ctop(zw, z2, n, n) - cbot(z1, zw, n, n)
                    + p[n] * q[n] * (-dtop(zw, z2, n, n) + dtop(z1, zw, n, n)))
        if case == "below":
            return -cbot(z1, z2, r, s) + p[t] * q[b] * dbot(z1, z2, r, s)
        return ctop(z1, z2, r, s) - p[t] * q[b] * dtop(z1, z2, r, s)

    pa = T(z1, z2, r, s)
    qa = R(z1, z2, r, s)
    if which == 1:
        return (a_rs / eta[s]) * (p[t] * pa + q[b] * qa + psi15())
    if which == 2:
        return (a_rs * eta[r]) * (p[t] * pa + q[b] * qa - psi15())
    if which == 3:
        return (a_rs * (eta[r] / eta[s])) * (p[t] * (-pa) + q[b] * qa + psi34())
    if which == 4:
        return a_rs * (p[t] * (-pa) + q[b] * qa - psi34())
    # which == 5
    if case == "match":
        n = r
        ln = m.section.thickness[n]
        kk = complex(0.0, om.omega) * om.zeta_bg[n] * MU0
        pq = p[n] * q[n]
        psi5 = (pq * (np.exp(-eta[n] * (2 * ln - (z2 - zw))) + np.exp(-eta[n] * (2 * ln - (zw - z1))))
                - (np.exp(-eta[n] * (z2 - zw)) + np.exp(-eta[n] * (zw - z1)))
                + 2 * kk * ((1 - pq * np.exp(-2 * eta[n] * ln)) / (lam * lam)))
        return (a_rs / eta[s]) * (p[t] * pa + q[b] * qa + psi5)
    return (a_rs / eta[s]) * (p[t] * pa + q[b] * qa + psi15())


def _a_matrix(om, eta, ex, p, q, r, s, sigma):
    """``GetAnn`` = A[r, s] of ``CalculateA1``/``CalculateASigma``
    (``PlanCalculator.cs:171-218``)."""
    tops = om.model.section.layer_tops()
    t, b = min(r, s), max(r, s)
    chain = propagator_chain(tops, eta, ex, p, q, t, b)
    if sigma and r > s:
        return (om.zeta_bg[r] / om.zeta_bg[s]) * chain
    return chain


def vtp_scalars_for_item(om, hankel, rho, lam, trans, kind):
    """``PlanCalculator.CalculateForE/H`` + ``NormalizeAndPerformHankel`` for
    one plan item; ``trans``: list of (z_receiver, z1, z2) per anomaly layer.
    Returns dict I -> [n_trans, n_rho] (E: 1..5, H: 1..4)."""
    m = om.model
    tops, thick = m.section.layer_tops(), m.section.thickness
    eta, ex = layer_eta_exp(om, lam)
    p1, q1, ps, qs = reflections(om, eta, ex)
    two_pi = 2 * np.pi
    need = (1, 2, 3, 4, 5) if kind == "E" else (1, 2, 3, 4)
    out = {k: np.empty((len(trans), rho.size), np.complex128) for k in need}
    for n_t, (zw, z1, z2) in enumerate(trans):
        r = corresponding_layer(tops, thick, zw)
        s = corresponding_layer(tops, thick, z1 + (z2 - z1) / 2)
        a1 = _a_matrix(om, eta, ex, p1, q1, r, s, False)
        a_s = _a_matrix(om, eta, ex, ps, qs, r, s, True)
        if kind == "E":
            zeta_rc2 = 2 * om.zeta_bg[r]
            i_omega_mu0 = complex(0.0, om.omega) * MU0
            u = {1: _vtp_u(om, eta, ex, p1, q1, a1, zw, z1, z2, r, s, 1, lam) * (i_omega_mu0 / 2),
                 2: _vtp_u(om, eta, ex, ps, qs, a_s, zw, z1, z2, r, s, 2, lam) / zeta_rc2,
                 3: _vtp_u(om, eta, ex, ps, qs, a_s, zw, z1, z2, r, s, 3, lam) * (lam / zeta_rc2),
                 4: _vtp_u(om, eta, ex, ps, qs, a_s, zw, z1, z2, r, s, 4, lam) * (-lam / zeta_rc2),
                 5: _vtp_u(om, eta, ex, ps, qs, a_s, zw, z1, z2, r, s, 5, lam) * ((lam * lam) / zeta_rc2)}
            for k in need:
                hank = hankel.h0 if k in (3, 4) else hankel.h1
                fr = hankel.convolve(hank, u[k], rho.size)
                out[k][n_t] = (-fr if k == 1 else fr) / (two_pi * rho)
        else:
            u11 = _vtp_u(om, eta, ex, p1, q1, a1, zw, z1, z2, r, s, 1, lam) * lam
            u31 = _vtp_u(om, eta, ex, p1, q1, a1, zw, z1, z2, r, s, 3, lam)
            u1s = _vtp_u(om, eta, ex, ps, qs, a_s, zw, z1, z2, r, s, 1, lam) * lam
            u4s = _vtp_u(om, eta, ex, ps, qs, a_s, zw, z1, z2, r, s, 4, lam)
            den = 2 * two_pi * rho
            out[1][n_t] = -hankel.convolve(hankel.h1, u31, rho.size) / den
            out[2][n_t] = -hankel.convolve(hankel.h1, u4s, rho.size) / den
            out[3][n_t] = -hankel.convolve(hankel.h0, u1s, rho.size) / den
            out[4][n_t] = hankel.convolve(hankel.h0, u11, rho.size) / den
    return out


def _zero_rho(rho, scal, kind, step):
    """``CalculateZeroRhoForE/H`` (``ScalarMathUtils.cs:33-87``): prepend
    rho = 0 with I1 = I2 (= I5) = 0 and I3, I4 extrapolated from the next
    two radii."""
    a2 = step * step
    out = {}
    for k, v in scal.items():
        if k in (3, 4):
            first = (v[:, 1] * a2 - v[:, 2]) / (a2 - 1)
        else:
            first = np.zeros(v.shape[0], np.complex128)
        out[k] = np.concatenate([first[:, None], v], axis=1)
    return np.concatenate([[0.0], rho]), out


def level_scalars(om, level, kind, n_hankels=10, hankel=None):
    hankel = hankel or Hankel()
    m = om.model
    items, add_zero = level_plan(m, level, n_hankels, hankel)
    trans = [(level.z, m.layer_depth[k], m.layer_depth[k] + m.layer_thickness[k]) for k in range(m.nz)]
    per_item = []
    rhos = []
    for i, (rho, lam) in enumerate(items):
        sc = vtp_scalars_for_item(om, hankel, rho, lam, trans, kind)
        if i == 0 and add_zero:
            rho, sc = _zero_rho(rho, sc, kind, hankel.rho_step())
        per_item.append(sc)
        rhos.append(rho)
    return combine([(rhos[i], None) for i in range(len(items))], per_item)


# ------------------------------------------------------------------ level tensor

# QSigns (QSign.cs:31-39)
Q_E = {
    ("x", False): {"xx": 1, "yy": -1, "zz": -1, "xy": -1, "xz": 1, "yz": 1, "zx": 1, "zy": 1},
    ("y", False): {"xx": -1, "yy": 1, "zz": -1, "xy": -1, "xz": 1, "yz": 1, "zx": 1, "zy": 1},
    ("x", True): {"xx": 1, "yy": -1, "zz": -1, "xy": 1, "xz": -1, "yz": 1, "zx": -1, "zy": 1},
    ("y", True): {"xx": -1, "yy": 1, "zz": -1, "xy": 1, "xz": 1, "yz": -1, "zx": 1, "zy": -1},
}
Q_H = {
    ("x", False): {"xx": -1, "xy": -1, "yx": 1, "xz": 1, "yz": 1, "zx": 1, "zy": 1},
    ("y", False): {"xx": -1, "xy": 1, "yx": -1, "xz": 1, "yz": 1, "zx": 1, "zy": 1},
    ("x", True): {"xx": 1, "xy": -1, "yx": 1, "xz": 1, "yz": -1, "zx": 1, "zy": -1},
    ("y", True): {"xx": 1, "xy": 1, "yx": -1, "xz": 1, "yz": 1, "zx": -1, "zy": 1},
}
# AddToQBuffAlong{X,Y}{Electric,Magnetic} (GreenTensorCalculator.cs:505-552):
# component -> (integral factor, scalar)
SRC_E = {
    "x": {"xx": ("D2", 1), "yy": ("D2", 2), "zz": ("D2", 5), "xy": ("D3", 2), "yz": ("D1", 3), "zy": ("D1", 4)},
    "y": {"xx": ("D2", 2), "yy": ("D2", 1), "zz": ("D2", 5), "xy": ("D3", 1), "xz": ("D1", 3), "zx": ("D1", 4)},
}
SRC_H = {
    "x": {"xx": ("D3", 2), "yx": ("D2", 1), "xy": ("D2", 2), "xz": ("D1", 3), "zx": ("D1", 4)},
    "y": {"yx": ("D2", 2), "xy": ("D2", 1), "xx": ("D3", 1), "yz": ("D1", 3), "zy": ("D1", 4)},
}


def level_events(m, radii, level):
    """Every face integration of ``RunAlongX``/``RunAlongY`` over the offsets
    i in [-Nx+1, Nx], j in [-Ny+1, Ny] with the level's shift
    (``AtoOLevelGreenTensorCalculator.cs:82-126``, ``GreenTensorCalculator.cs:166-437``),
    with the cells (after ``TransformI/J``) each is added to."""
    nx, ny, dx, dy = m.nx, m.ny, m.dx, m.dy
    lx, rx, ly, ry = -nx + 1, nx, -ny + 1, ny
    xs, ys = -level.shift_x, -level.shift_y   # GetXShift() = -ShiftX

    def X(i):
        return dx * (i - 0.5) - xs

    def Y(j):
        return dy * (j - 0.5) - ys
    kn = {(i, j): knot(radii, X(i), Y(j)) for i in range(lx, rx + 1) for j in range(ly, ry + 1)}
    zx = {j: knot(radii, 0.0, Y(j)) for j in range(ly, ry + 1)}
    zy = {i: knot(radii, X(i), 0.0) for i in range(lx, rx + 1)}

    def ti(i):
        return 2 * nx + i if i < 0 else i

    def tj(j):
        return 2 * ny + j if j < 0 else j

    def cells_x(i, j):
        if j == ly:
            return [(ti(i), tj(ly), -1)]
        if j == ry:
            return [(ti(i), tj(ry - 1), 1)]
        return [(ti(i), tj(j - 1), 1), (ti(i), tj(j), -1)]

    def cells_y(i, j):
        if i == lx:
            return [(ti(lx), tj(j), -1)]
        if i == rx:
            return [(ti(rx - 1), tj(j), 1)]
        return [(ti(i - 1), tj(j), 1), (ti(i), tj(j), -1)]

    for j in range(ly, ry + 1):
        y = Y(j)
        for i in range(lx, rx):
            x1, x2 = X(i), X(i + 1)
            if x1 > 0 and x2 > 0:
                yield "x", False, cells_x(i, j), integrate(radii, kn[i, j], kn[i + 1, j], x1, x2, y)
            elif x1 < 0 and x2 < 0:
                yield "x", True, cells_x(i, j), integrate(radii, kn[i + 1, j], kn[i, j], -x2, -x1, y)
            else:
                yield "x", True, cells_x(i, j), integrate(radii, zx[j], kn[i, j], 0.0, -x1, y)
                yield "x", False, cells_x(i, j), integrate(radii, zx[j], kn[i + 1, j], 0.0, x2, y)
    for i in range(lx, rx + 1):
        x = X(i)
        for j in range(ly, ry):
            y1, y2 = Y(j), Y(j + 1)
            if y1 > 0 and y2 > 0:
                yield "y", False, cells_y(i, j), integrate(radii, kn[i, j], kn[i, j + 1], y1, y2, x)
            elif y1 < 0 and y2 < 0:
                yield "y", True, cells_y(i, j), integrate(radii, kn[i, j + 1], kn[i, j], -y2, -y1, x)
            else:
                yield "y", True, cells_y(i, j), integrate(radii, zy[i], kn[i, j], 0.0, -y1, x)
                yield "y", False, cells_y(i, j), integrate(radii, zy[i], kn[i, j + 1], 0.0, y2, x)


def level_realspace(om, level, kind, n_hankels=10):
    """Real-space level tensor: dict component -> [2Nx, 2Ny, Nz] (offset index
    Nx and Ny never written)."""
    m = om.model
    radii, scal = level_scalars(om, level, kind, n_hankels)
    segs = segments(radii, scal)
    comps = E_COMPS if kind == "E" else H_COMPS
    qsig = Q_E if kind == "E" else Q_H
    src = SRC_E if kind == "E" else SRC_H
    out = {c: np.zeros((2 * m.nx, 2 * m.ny, m.nz), np.complex128) for c in comps}
    for direction, symm, cells, parts in level_events(m, radii, level):
        qs = qsig[direction, symm]
        for c, (fac, sc) in src[direction].items():
            sa, sb = segs[sc]
            val = np.zeros(m.nz, np.complex128)
            for seg, f in parts:
                da, db = f[fac]
                val = val + da * sa[seg] + db * sb[seg]
            for (i, j, sign) in cells:
                out[c][i, j] += (sign * qs[c]) * val
    return out


def level_tensor(om, level, kind, n_hankels=10):
    """Spectral level tensor (``AtoOCalculator.PerformGreenTensorFft``):
    dict component -> [2Nx, 2Ny, Nz]."""
    return {c: np.fft.fft2(v, axes=(0, 1)) for c, v in level_realspace(om, level, kind, n_hankels).items()}


# ------------------------------------------------------------------ fields and responses

def anomaly_field(om, G, jq, kind):
    """``ToOCalculator.CalculateAnomalyField`` (``ToOCalculator.cs:21-125``):
    field [Nx, Ny, 3] at the level from jQ [Nx*Ny*3*Nz]."""
    m = om.model
    nx, ny, nz = m.nx, m.ny, m.nz
    buf = np.zeros((2 * nx, 2 * ny, 3, nz), np.complex128)
    buf[:nx, :ny] = jq.reshape(nx, ny, 3, nz)
    X = np.fft.fft2(buf, axes=(0, 1))
    sx, sy, sz = X[:, :, 0], X[:, :, 1], X[:, :, 2]

    def g(c, s):
        # ZgemvAtoO: sum over the transmitter layers, no conjugation
        return np.sum(G[c] * s, axis=-1)
    out = np.empty((2 * nx, 2 * ny, 3), np.complex128)
    if kind == "E":
        out[..., 0] = g("xx", sx) + g("xy", sy) + g("xz", sz)
        out[..., 1] = g("xy", sx) + g("yy", sy) + g("yz", sz)
        out[..., 2] = g("zx", sx) + g("zy", sy) + g("zz", sz)
    else:
        out[..., 0] = -g("xx", sx) - g("xy", sy) - g("xz", sz)
        out[..., 1] = g("yx", sx) + g("xx", sy) + g("yz", sz)
        out[..., 2] = -g("zx", sx) + g("zy", sy)
    back = np.fft.ifft2(out, axes=(0, 1)) * (4 * nx * ny)   # unnormalised backward
    back = back / (4.0 * nx * ny)                          # Zscal by 1/(4 Nx Ny)
    return back[:nx, :ny]


def normal_fields(om, z, pol):
    """E and H of the plane wave at depth z for one polarisation
    (``Mt3DForwardSolver.CalculateNormalFieldE/H``, ``:300-337``)."""
    e = _mt.plane_wave_e(om, z)
    h = _mt.plane_wave_h(om, z)
    if pol == 0:
        return np.array([e, 0, 0], complex), np.array([0, h, 0], complex)
    return np.array([0, e, 0], complex), np.array([-h, 0, 0], complex)


def impedance(e1, e2, h1, h2):
    """``ResponseFunctionsCalculator.CalculateTensor`` (``:36-51``) on
    [..., 3] fields of the two polarisations: Z [..., 2, 2]."""
    det = h1[..., 0] * h2[..., 1] - h2[..., 0] * h1[..., 1]
    hi11 = h2[..., 1] / det
    hi12 = -h2[..., 0] / det
    hi21 = -h1[..., 1] / det
    hi22 = h1[..., 0] / det
    z = np.empty(det.shape + (2, 2), np.complex128)
    z[..., 0, 0] = e1[..., 0] * hi11 + e2[..., 0] * hi21
    z[..., 0, 1] = e1[..., 0] * hi12 + e2[..., 0] * hi22
    z[..., 1, 0] = e1[..., 1] * hi11 + e2[..., 1] * hi21
    z[..., 1, 1] = e1[..., 1] * hi12 + e2[..., 1] * hi22
    return z


def rho_phase(z, omega, degrees=True, reverse_sign=False):
    """``CalculateApparentResistivity`` and ``ProcessPhase``
    (``PlainTextExporter.cs:360-420``)."""
    rho = np.abs(z) ** 2 / (omega * MU0)
    ph = np.angle(z)
    if degrees:
        ph = ph * (180 / np.pi)
    if reverse_sign:
        ph = -ph
    return rho, ph


def level_responses(om, level, jq_x, jq_y, n_hankels=10):
    """Full fields of both polarisations at the level's cell centres and the
    impedance, apparent resistivity and phase: dict of arrays."""
    ge = level_tensor(om, level, "E", n_hankels)
    gh = level_tensor(om, level, "H", n_hankels)
    out = {}
    full = {}
    for pol, jq in ((0, jq_x), (1, jq_y)):
        en, hn = normal_fields(om, level.z, pol)
        ea = anomaly_field(om, ge, jq, "E")
        ha = anomaly_field(om, gh, jq, "H")
        out["anomaly_e%d" % pol] = ea
        out["anomaly_h%d" % pol] = ha
        full["e%d" % pol] = ea + en
        full["h%d" % pol] = ha + hn
    z = impedance(full["e0"], full["e1"], full["h0"], full["h1"])
    rho, ph = rho_phase(z, om.omega)
    out.update(full)
    out.update({"z": z, "rho": rho, "phase": ph})
    return out
