"""Oracle (TEST INFRASTRUCTURE ONLY, see ``oracle/__init__.py``): anomaly-to-anomaly (AtoA) Green tensor of the layered background,
restated in numpy complex128 from the reference.

Pipeline (``Extreme.Cartesian/Forward/AtoA/AtoAGreenTensorCalculatorComponent.cs:82-279``):

1. radius plan: log-spaced radii from ``min(dx,dy)/2`` to the mesh diagonal,
   ``NumberOfHankels`` shifted copies (``Green/Scalar/ScalarPlansCreater.cs:102-176``,
   ``Green/Scalar/ScalarPlan.cs:450-481``);
2. scalars ``I1..I5`` per transceiver pair: vertical wavenumbers, layer
   reflection recursions, propagators, kernels ``U1..U5`` and the ndec=40
   digital Hankel filter (``Green/Scalar/Impl/PlanCalculatorFast.cs:80-318``,
   ``Green/Scalar/Impl/VolumeToVolumeCalculatorUFast.cs:34-337``,
   ``Native/Native.Matrix/green_scalar.c:30-386``,
   ``Green/Scalar/Impl/ScalarMathUtils.cs:99-263``,
   ``Green/Scalar/Impl/HankelCoefficients.cs:103-118``);
3. merge of the plan items by radius, linear segments per radius interval
   (``Green/Scalar/Impl/InnerResultsCombiner.cs:19-61``,
   ``Green/Tensor/Impl/ScalarSegments.cs:80-128``);
4. integration of the segments over the cell faces along x and y
   (``Green/Tensor/Impl/GreenTensorCalculator.cs:166-552``,
   ``Green/Tensor/Impl/IntegralFactors.cs:17-30``, ``Green/Tensor/Impl/QSign.cs:31-39``);
5. mirroring into the ``2Nx x 2Ny`` circulant grid
   (``Green/Tensor/Impl/GreenTensorFftPopulator.cs:170-273``);
6. unnormalised forward 2-D FFT of every block entry (FFTW sign -1).

The summation order of the face integrals differs from the reference (sparse
matrix products instead of per-face loops); everything else follows the
reference's order of operations.
"""
import os

import numpy as np
import scipy.sparse as sp

MU0 = 4.0 * np.pi * 1.0e-7

_HERE = os.path.dirname(os.path.abspath(__file__))
_HANKEL = os.path.join(_HERE, "..", "extreme_gb300", "data", "hankel_ndec40.npz")


# --------------------------------------------------------------------------
# Hankel filter and radius plan
# --------------------------------------------------------------------------

class Hankel:
    """ndec=40 filter: 431 taps, l1=-300, l2=130
    (``HankelCoefficients.cs:37,67-76``)."""

    def __init__(self):
        d = np.load(_HANKEL)
        self.h0 = d["h0"]
        self.h1 = d["h1"]
        self.ndec = 40
        self.l1 = -300
        self.l2 = 130

    def rho_step(self):
        """``(float)Math.Pow(10, 1 / _ndec)`` with a float ``_ndec``: the
        exponent is a float division and the result is rounded to float
        (``HankelCoefficients.cs:67``)."""
        e = float(np.float32(1.0) / np.float32(self.ndec))
        return float(np.float32(10.0 ** e))

    def n_lambda(self, n_rho):
        return self.h0.size + n_rho

    def n1(self):
        return 0 - self.l2

    def convolve(self, hank, fk, n_rho):
        """``ConvoluteWithFast``: fr[i] = sum_j rev(hank)[j] * fk[i + j]
        (``HankelCoefficients.cs:103-118``; ``green_scalar.c:43-55``)."""
        rev = hank[::-1]
        shift0 = -(self.l1 + self.n1()) - rev.size + 1
        assert shift0 == 0
        win = np.lib.stride_tricks.sliding_window_view(fk, rev.size, axis=-1)[..., :n_rho, :]
        return win @ rev


def rho_from_min(rho_min, rho_max, step):
    """``ScalarPlansCreater.CreateRhoFromMin`` (``ScalarPlansCreater.cs:142-157``)."""
    out = []
    r = rho_min
    while r <= rho_max:
        out.append(r)
        r *= step
    out.append(r)
    return np.array(out)


def rho_from_max(rho_min, rho_max, step):
    """``ScalarPlansCreater.CreateRhoFromMax`` (``ScalarPlansCreater.cs:159-176``)."""
    out = []
    r = rho_max
    while r >= rho_min:
        out.append(r)
        r /= step
    out.append(r)
    return np.array(out[::-1])


def lambdas_for(hankel, rho):
    """``ScalarPlan.CalculateLambdasForLog10`` (``ScalarPlan.cs:460-481``)."""
    n = hankel.n_lambda(rho.size)
    k = np.empty(n)
    step = hankel.rho_step()
    n1 = hankel.n1()
    n2 = n - 1 - hankel.l2
    k[-n1] = 1.0 / rho[0]
    for i in range(-n1 + 1, n2 - n1 + 1):
        k[i] = k[i - 1] / step
    for i in range(-n1 - 1, -1, -1):
        k[i] = k[i + 1] * step
    return k


def anomaly_plan(dx, dy, nx, ny, n_hankels, hankel=None):
    """Radius plan of the AtoA tensor (``ScalarPlansCreater.cs:102-140,360-380``):
    list of (rho, lambdas) plan items."""
    hankel = hankel or Hankel()
    half1, half2 = dx / 2.0, dy / 2.0
    rho_min = min(half1, half2)
    max_x = nx * dx - half1
    max_y = ny * dy - half2
    rho_max = np.sqrt(max_x * max_x + max_y * max_y)
    step = hankel.rho_step()
    n = abs(n_hankels)
    rho1 = rho_from_min(rho_min, rho_max, step)
    r2, r1 = rho1[-1], rho1[-2]
    lin = (r2 - r1) / n
    items = [rho1]
    for i in range(1, n):
        items.append(rho_from_max(rho_min, r2 - i * lin, step))
    return [(rho, lambdas_for(hankel, rho)) for rho in items]


# --------------------------------------------------------------------------
# Scalars I1..I5
# --------------------------------------------------------------------------

def _section_arrays(om):
    m = om.model
    tops = m.section.layer_tops()
    thick = m.section.thickness
    return tops, thick, om.zeta_bg


def corresponding_layer(tops, thick, depth):
    """``ScalarMathUtils.DetermineCorrespondingBackgroundLayer``
    (``ScalarMathUtils.cs:15-31``)."""
    prev = tops[0]
    for k in range(len(thick)):
        d1, d2 = prev, prev + thick[k]
        if d1 <= depth < d2:
            return k
        prev = d2
    raise ValueError("depth %r is not within the 1-D section" % depth)


def layer_eta_exp(om, lam):
    """``CalculateEta``/``CalculateExp`` (``PlanCalculatorFast.cs:203-233``,
    ``green_scalar.c:30-41``): eta[k,m] = sqrt(lam^2 - i*omega*mu0*zeta_k),
    exp[k,m] = exp(-2*thick_k*eta[k,m])."""
    tops, thick, zb = _section_arrays(om)
    eta = np.empty((len(zb), lam.size), np.complex128)
    ex = np.empty_like(eta)
    for k in range(len(zb)):
        value = eta_shift(om.omega, zb[k])
        eta[k] = np.sqrt(real_minus_complex(lam * lam, value))
        ex[k] = np.exp(eta[k] * (-2.0 * thick[k]))
    return eta, ex


def eta_shift(omega, zeta):
    """``iOmega * zeta * Mu0`` as the C# complex arithmetic forms it
    (``PlanCalculatorFast.cs:222-229``)."""
    return complex(0.0, omega) * zeta * MU0


def real_minus_complex(x, value):
    """C99 ``double - double complex`` (``green_scalar.c:33``): the real
    operand is not widened, so the imaginary part is ``-Im(value)`` (a
    negative zero when ``Im(value) == +0``, which selects the lower branch of
    ``csqrt`` for the air layer at ``lambda < omega/c``)."""
    out = np.empty(np.shape(x), np.complex128)
    out.real = x - value.real
    out.imag = -value.imag
    return out


def p_recursion(eta, ex, p1, alpha):
    """``CalculatePBelow1`` (``PlanCalculatorFast.cs:266-280``)."""
    p = np.zeros_like(eta)
    p[1] = p1
    for k in range(1, eta.shape[0] - 1):
        pexp = p[k] * ex[k]
        alpha_eta = alpha[k] * (eta[k] / eta[k + 1])
        part = alpha_eta * ((pexp - 1) / (pexp + 1))
        p[k + 1] = (1 + part) / (1 - part)
    return p


def q_recursion(eta, ex, beta):
    """``CalculateQ`` (``PlanCalculatorFast.cs:292-318``)."""
    q = np.zeros_like(eta)
    n = eta.shape[0] - 1
    part = beta[n] * (eta[n] / eta[n - 1])
    q[n - 1] = (1 - part) / (1 + part)
    for k in range(n - 1, 1, -1):
        qexp = q[k] * ex[k]
        beta_eta = beta[k] * (eta[k] / eta[k - 1])
        part = beta_eta * ((qexp - 1) / (qexp + 1))
        q[k - 1] = (1 + part) / (1 - part)
    return q


def reflections(om, eta, ex):
    """P/Q for the "1" and "sigma" modes (``PlanCalculatorFast.cs:236-318``,
    ``Green/Scalar/Impl/AlphaBeta.cs:344-362``)."""
    zb = om.zeta_bg
    L = len(zb)
    ones = np.ones(L, np.complex128)
    alpha_s = np.zeros(L, np.complex128)
    beta_s = np.zeros(L, np.complex128)
    for k in range(L - 1):
        alpha_s[k] = zb[k + 1] / zb[k]
    for k in range(1, L):
        beta_s[k] = zb[k - 1] / zb[k]
    p1 = p_recursion(eta, ex, (eta[1] - eta[0]) / (eta[1] + eta[0]), ones)
    q1 = q_recursion(eta, ex, ones)
    ps = p_recursion(eta, ex, (zb[0] * eta[1] - zb[1] * eta[0]) / (zb[0] * eta[1] + zb[1] * eta[0]), alpha_s)
    qs = q_recursion(eta, ex, beta_s)
    return p1, q1, ps, qs


def propagator_chain(tops, eta, ex, p, q, lo, hi):
    """``A[lo, hi]`` of ``CalculateA`` (``PlanCalculatorFast.cs:160-200``):
    A[hi,hi] = 1/(eta_hi (1 - P Q exp)), then multiplied up to layer lo."""
    a = 1.0 / (eta[hi] * (1 - p[hi] * q[hi] * ex[hi]))
    for k in range(hi - 1, lo - 1, -1):
        dk1 = tops[k + 1]
        f = ((1 + p[k + 1]) / (1 + p[k] * ex[k])) * np.exp((eta[k + 1] - eta[k]) * dk1)
        a = f * a
    return a


def _lin(*terms):
    acc = 0.0
    for c, v in terms:
        acc = acc + c * v
    return acc


def exp_sums(eta, r, s, t, b, dt, db1, r1, r2, s1, s2):
    """``CalculateT/R/CTop/CBot/DTop/DBot`` (``green_scalar.c:86-386``):
    the four-term exponential sums of the vertical integrals."""
    er, es, et, eb = eta[r], eta[s], eta[t], eta[b]

    def e(z):
        return np.exp(z)

    # The six sums are formed for every (transceiver, lambda), as the
    # reference's C does (green_scalar.c:86-386); the ones that the
    # transceiver's layer case does not use can overflow to inf, and their
    # four-term differences become inf - inf = NaN. Those entries are never
    # read (scalars_for_item picks the sums of its case), so overflow and
    # invalid operations are masked here explicitly, for all six sums.
    with np.errstate(over="ignore", invalid="ignore"):
        T = (e(_lin((-r1, er), (-s1, es), (2 * dt, et))) - e(_lin((-r1, er), (-s2, es), (2 * dt, et)))
             - e(_lin((-r2, er), (-s1, es), (2 * dt, et))) + e(_lin((-r2, er), (-s2, es), (2 * dt, et))))
        R = (e(_lin((-2 * db1, eb), (s2, es), (r2, er))) - e(_lin((-2 * db1, eb), (s1, es), (r2, er)))
             - e(_lin((-2 * db1, eb), (s2, es), (r1, er))) + e(_lin((-2 * db1, eb), (s1, es), (r1, er))))
        ctop = (e(_lin((-s1, es), (r2, er))) - e(_lin((-s2, es), (r2, er)))
                - e(_lin((-s1, es), (r1, er))) + e(_lin((-s2, es), (r1, er))))
        cbot = (e(_lin((-r1, er), (s2, es))) - e(_lin((-r1, er), (s1, es)))
                - e(_lin((-r2, er), (s2, es))) + e(_lin((-r2, er), (s1, es))))
        first = _lin((-2 * db1, eb), (2 * dt, et))
        dtop, dbot = _d_sums(e, first, es, er, s1, s2, r1, r2)
    return T, R, ctop, cbot, dtop, dbot


def _d_sums(e, first, es, er, s1, s2, r1, r2):
    dtop = (e(first + s2 * es + (-r1) * er) - e(first + s1 * es + (-r1) * er)
            - e(first + s2 * es + (-r2) * er) + e(first + s1 * es + (-r2) * er))
    dbot = (e(first + (-s1) * es + r2 * er) - e(first + (-s2) * es + r2 * er)
            - e(first + (-s1) * es + r1 * er) + e(first + (-s2) * es + r1 * er))
    return dtop, dbot


def scalars_for_item(om, hankel, rho, lam, trans, need):
    """``PlanCalculatorFast.CalculateForE`` + ``NormalizeAndPerformHankelFast``
    for one plan item and a list of transceivers.

    ``trans``: list of (r1, r2, s1, s2) receiver/transmitter layer bounds.
    ``need``: subset of {1,2,3,4,5}. Returns dict I -> [n_trans, n_rho].
    """
    tops, thick, zb = _section_arrays(om)
    eta, ex = layer_eta_exp(om, lam)
    p1, q1, ps, qs = reflections(om, eta, ex)
    i_omega_mu0 = complex(0.0, om.omega) * MU0
    out = {k: np.empty((len(trans), rho.size), np.complex128) for k in need}
    two_pi = 2 * np.pi
    for n_t, (r1, r2, s1, s2) in enumerate(trans):
        zwork = r1 + (r2 - r1) / 2
        r = corresponding_layer(tops, thick, zwork)
        s = corresponding_layer(tops, thick, s1 + (s2 - s1) / 2)
        t, b = min(r, s), max(r, s)
        dt, db1 = tops[t], tops[b + 1]
        T, R, ctop, cbot, dtop, dbot = exp_sums(eta, r, s, t, b, dt, db1, r1, r2, s1, s2)
        if s1 < zwork < s2:
            case = "match"
        elif zwork >= s2:
            case = "below"
        else:
            case = "above"

        def psi1(p, q):
            if case == "match":
                tau = r2 - r1
                n = r
                dn1 = tops[n + 1] - tops[n]
                part1 = tau * eta[n] - (1 - np.exp(-eta[n] * tau))
                part2 = p[n] * q[n] * ((tau * eta[n] + 1) * np.exp(-2 * eta[n] * dn1)
                                       - np.exp(-2 * eta[n] * dn1 + eta[n] * tau))
                return 2 * (part1 - part2)
            if case == "below":
                return cbot + p[t] * q[b] * dbot
            return ctop + p[t] * q[b] * dtop

        def psi3(p, q):
            if case == "match":
                return np.zeros(lam.size, np.complex128)
            if case == "below":
                return -cbot + p[t] * q[b] * dbot
            return ctop - p[t] * q[b] * dtop

        def special(p, q, psign, psisign, psi):
            return psign * p[t] * T + q[b] * R + psisign * psi

        ann_factor = 1 / (eta[r] * eta[s])
        u = {}
        if 1 in need:
            ann = propagator_chain(tops, eta, ex, p1, q1, t, b)
            u[1] = ann * ann_factor * special(p1, q1, 1, 1, psi1(p1, q1))
        chain_s = propagator_chain(tops, eta, ex, ps, qs, t, b)
        ann_s = (zb[r] / zb[s]) * chain_s if r > s else chain_s
        if 2 in need:
            u[2] = ann_s * special(ps, qs, 1, -1, psi1(ps, qs))
        if 3 in need:
            u[3] = ann_s * (1 / eta[s]) * special(ps, qs, -1, 1, psi3(ps, qs))
        if 4 in need:
            u[4] = ann_s * (1 / eta[r]) * special(ps, qs, -1, -1, psi3(ps, qs))
        if 5 in need:
            if case == "match":
                n = r
                tau = r2 - r1
                ln = thick[n]
                kk = complex(0.0, om.omega) * zb[n] * MU0
                pq = ps[n] * qs[n]
                part1 = -(1 - np.exp(-eta[n] * tau))
                part2 = pq * (np.exp(-eta[n] * (2 * ln - tau)) - np.exp(-2 * eta[n] * ln))
                part3 = (kk / (lam * lam)) * (1 - pq * np.exp(-2 * eta[n] * ln)) * tau * eta[n]
                psi5 = 2 * (part1 + part2 + part3)
                u[5] = (ann_s * ann_factor) * (ps[t] * T + qs[b] * R + psi5)
            else:
                u[5] = ann_s * ann_factor * special(ps, qs, 1, 1, psi1(ps, qs))
        # NormalizeBeforeHankelForE (ScalarMathUtils.cs:243-263)
        zeta_rc2 = 2 * zb[r]
        if 1 in need:
            u[1] = u[1] * (i_omega_mu0 / 2)
        if 2 in need:
            u[2] = u[2] / zeta_rc2
        if 3 in need:
            u[3] = u[3] * (lam / zeta_rc2)
        if 4 in need:
            u[4] = u[4] * (-lam / zeta_rc2)
        if 5 in need:
            u[5] = u[5] * ((lam * lam) / zeta_rc2)
        # CalculateHankelForEFast + NormalizeAfterHankelForE (ScalarMathUtils.cs:189-241)
        for k in need:
            hank = hankel.h0 if k in (3, 4) else hankel.h1
            fr = hankel.convolve(hank, u[k], rho.size)
            if k == 1:
                fr = -fr / (two_pi * rho)
            else:
                fr = fr / (two_pi * rho)
            out[k][n_t] = fr
    return out


def combine(items, per_item):
    """``InnerResultsCombiner`` + ``ScalarPlan.GetSortedRho``: merge the plan
    items' radii into one sorted list (``InnerResultsCombiner.cs:19-61``,
    ``ScalarPlan.cs:439-448``)."""
    keys = {}
    for i, (rho, _) in enumerate(items):
        for j, r in enumerate(rho):
            if r not in keys:
                keys[r] = (i, j)
    radii = np.sort(np.concatenate([rho for rho, _ in items]))
    uniq = sorted(keys)
    if len(uniq) != radii.size:
        raise ValueError("duplicate radii across plan items")
    comps = per_item[0].keys()
    merged = {}
    for c in comps:
        ntr = per_item[0][c].shape[0]
        arr = np.empty((ntr, len(uniq)), np.complex128)
        for k, r in enumerate(uniq):
            i, j = keys[r]
            arr[:, k] = per_item[i][c][:, j]
        merged[c] = arr
    return radii, merged


def segments(radii, scalars):
    """``ScalarSegments.CalculateScalarSegment`` (``ScalarSegments.cs:86-128``):
    I(rho) = A*rho + B on each radius interval. Returns c -> (A, B) with shapes
    [n_seg, n_trans]."""
    s = radii[:-1]
    u = radii[1:]
    div = u - s
    out = {}
    for c, v in scalars.items():
        a = (v[:, 1:] - v[:, :-1]) / div[None, :]
        b = v[:, :-1] - a * s[None, :]
        out[c] = (a.T.copy(), b.T.copy())
    return out


# --------------------------------------------------------------------------
# Transceivers and the scalar step for one tensor half
# --------------------------------------------------------------------------

def asym_transceivers(model):
    """``TranceiverUtils.Combine``: receiver-major, index ``rc*Nz + tr``
    (``Model/TranceiverUtils.cs:55-63``)."""
    d, t = model.layer_depth, model.layer_thickness
    return [(d[rc], d[rc] + t[rc], d[tr], d[tr] + t[tr])
            for rc in range(model.nz) for tr in range(model.nz)]


def symm_transceivers(model):
    """``TranceiverUtils.CombineSymm``: transmitter-major with ``rc <= tr``,
    index ``tr*(tr+1)/2 + rc`` (``Model/TranceiverUtils.cs:65-74``)."""
    d, t = model.layer_depth, model.layer_thickness
    return [(d[rc], d[rc] + t[rc], d[tr], d[tr] + t[tr])
            for tr in range(model.nz) for rc in range(tr + 1)]


def compute_scalars(om, n_hankels, trans, need, hankel=None):
    hankel = hankel or Hankel()
    m = om.model
    items = anomaly_plan(m.dx, m.dy, m.nx, m.ny, n_hankels, hankel)
    per_item = [scalars_for_item(om, hankel, rho, lam, trans, need) for rho, lam in items]
    radii, merged = combine(items, per_item)
    return radii, merged


# --------------------------------------------------------------------------
# Face integration (GreenTensorCalculator.RunAlongX/RunAlongY)
# --------------------------------------------------------------------------

def integral_factors(s, u, rs, ru, v):
    """``IntegralFactors.Prepare`` (``IntegralFactors.cs:17-30``)."""
    if v == 0:
        d1a = (u * ru - s * rs) / 2
        d2a = 0.0
        d2b = 0.0
    else:
        lg = np.log((u + ru) / (s + rs))
        d1a = (u * ru - s * rs + v * v * lg) / 2
        d2a = -(u - s) * v
        d2b = -(v * lg)
    return {"D1": (d1a, u - s), "D2": (d2a, d2b), "D3": (-(u * u - s * s) / 2, -(ru - rs))}


def knot(radii, x, y):
    """``PrepareKnot`` (``GreenTensorCalculator.cs:207-228``)."""
    r = np.sqrt(x * x + y * y)
    idx = int(np.searchsorted(radii, r, side="right")) - 1
    if idx == radii.size - 1:
        idx -= 1
    if idx < 0:
        idx = 0
    return idx, r


def integrate(radii, left, right, s, u, v):
    """``GreenTensorCalculator.Integrate`` (``GreenTensorCalculator.cs:367-411``):
    list of (segment index, factors) along one face line."""
    i1, rl = left
    i2, rr = right
    if i1 == i2:
        return [(i1, integral_factors(s, u, rl, rr, v))]
    out = []
    r1 = rl
    r2 = radii[i1 + 1]
    sj = s
    uj = np.sqrt(r2 * r2 - v * v)
    out.append((i1, integral_factors(sj, uj, r1, r2, v)))
    for i in range(i1 + 1, i2):
        r1 = r2
        r2 = radii[i + 1]
        sj = uj
        uj = np.sqrt(r2 * r2 - v * v)
        out.append((i, integral_factors(sj, uj, r1, r2, v)))
    sj = uj
    uj = u
    r1 = r2
    r2 = rr
    out.append((i2, integral_factors(sj, uj, r1, r2, v)))
    return out


# QSigns (QSign.cs:254-257): component -> sign
Q_ALONG_X = {"xx": 1, "yy": -1, "zz": -1, "xy": -1, "xz": 1, "yz": 1}
Q_ALONG_Y = {"xx": -1, "yy": 1, "zz": -1, "xy": -1, "xz": 1, "yz": 1}
Q_ALONG_X_SYMM = {"xx": 1, "yy": -1, "zz": -1, "xy": 1, "xz": -1, "yz": 1}
Q_ALONG_Y_SYMM = {"xx": -1, "yy": 1, "zz": -1, "xy": 1, "xz": 1, "yz": -1}

# AddToQBuffAlong{X,Y}Electric (GreenTensorCalculator.cs:505-528):
# component -> (integral factor, scalar)
SRC_ALONG_X = {"xx": ("D2", 1), "yy": ("D2", 2), "zz": ("D2", 5), "xy": ("D3", 2), "yz": ("D1", 3)}
SRC_ALONG_Y = {"xx": ("D2", 2), "yy": ("D2", 1), "zz": ("D2", 5), "xy": ("D3", 1), "xz": ("D1", 3)}


def face_events(model, radii):
    """Enumerate every face integration of ``RunAlongX``/``RunAlongY``
    (``GreenTensorCalculator.cs:254-361``) with the cells it is added to
    (``FillResultAlongX/Y``, ``:413-437``).

    Yields (direction, symm, [(i, j, sign)], [(seg, factors)]).
    """
    nx, ny = model.nx, model.ny
    dx, dy = model.dx, model.dy
    kn = {}
    for i in range(nx + 1):
        for j in range(ny + 1):
            kn[i, j] = knot(radii, dx * (i - 0.5), dy * (j - 0.5))
    zx = [knot(radii, 0.0, dy * (j - 0.5)) for j in range(ny + 1)]
    zy = [knot(radii, dx * (i - 0.5), 0.0) for i in range(nx + 1)]

    def cells_x(i, j):
        if j == 0:
            return [(i, 0, -1)]
        if j == ny:
            return [(i, ny - 1, 1)]
        return [(i, j - 1, 1), (i, j, -1)]

    def cells_y(i, j):
        if i == 0:
            return [(0, j, -1)]
        if i == nx:
            return [(nx - 1, j, 1)]
        return [(i - 1, j, 1), (i, j, -1)]

    for j in range(ny + 1):
        y = dy * (j - 0.5)
        for i in range(nx):
            x1 = dx * (i - 0.5)
            x2 = dx * (i + 0.5)
            if x1 > 0 and x2 > 0:
                yield "x", False, cells_x(i, j), integrate(radii, kn[i, j], kn[i + 1, j], x1, x2, y)
            elif x1 < 0 and x2 < 0:
                yield "x", True, cells_x(i, j), integrate(radii, kn[i + 1, j], kn[i, j], -x2, -x1, y)
            else:
                yield "x", True, cells_x(i, j), integrate(radii, zx[j], kn[i, j], 0.0, -x1, y)
                yield "x", False, cells_x(i, j), integrate(radii, zx[j], kn[i + 1, j], 0.0, x2, y)
    for i in range(nx + 1):
        x = dx * (i - 0.5)
        for j in range(ny):
            y1 = dy * (j - 0.5)
            y2 = dy * (j + 0.5)
            if y1 > 0 and y2 > 0:
                yield "y", False, cells_y(i, j), integrate(radii, kn[i, j], kn[i, j + 1], y1, y2, x)
            elif y1 < 0 and y2 < 0:
                yield "y", True, cells_y(i, j), integrate(radii, kn[i, j + 1], kn[i, j], -y2, -y1, x)
            else:
                yield "y", True, cells_y(i, j), integrate(radii, zy[i], kn[i, j], 0.0, -y1, x)
                yield "y", False, cells_y(i, j), integrate(radii, zy[i], kn[i, j + 1], 0.0, y2, x)


def integrate_tensor(model, radii, segs, comps):
    """Real-space tensor on the ``Nx x Ny`` quadrant for the components
    ``comps``; ``segs``: scalar index -> (A, B) [n_seg, block].

    Each cell value is the signed sum of its face integrals
    (``FillGreen``, ``GreenTensorCalculator.cs:460-497``), each face integral a
    sum over radius segments of ``D?A * I?A + D?B * I?B``
    (``AddToQBuffAlong{X,Y}Electric``, ``:505-528``). The weights are gathered
    into sparse (cell x segment) matrices per direction.
    """
    nx, ny = model.nx, model.ny
    nseg = radii.size - 1
    events = _cached_events(model, radii)
    res = {}
    for c in comps:
        acc = None
        for direction, src in (("x", SRC_ALONG_X), ("y", SRC_ALONG_Y)):
            if c not in src:
                continue
            qsr = Q_ALONG_X if direction == "x" else Q_ALONG_Y
            qss = Q_ALONG_X_SYMM if direction == "x" else Q_ALONG_Y_SYMM
            fac, scal = src[c]
            r_, c_, a_, b_ = [], [], [], []
            for d, symm, cells, parts in events:
                if d != direction:
                    continue
                qs = qss if symm else qsr
                for (i, j, sign) in cells:
                    w = sign * qs[c]
                    cell = i * ny + j
                    for seg, f in parts:
                        da, db = f[fac]
                        r_.append(cell)
                        c_.append(seg)
                        a_.append(w * da)
                        b_.append(w * db)
            wa = sp.csr_matrix((a_, (r_, c_)), shape=(nx * ny, nseg))
            wb = sp.csr_matrix((b_, (r_, c_)), shape=(nx * ny, nseg))
            sa, sb = segs[scal]
            term = wa @ sa + wb @ sb
            acc = term if acc is None else acc + term
        res[c] = np.asarray(acc).reshape(nx, ny, -1)
    return res


_EVENT_CACHE = {}


def _cached_events(model, radii):
    key = (model.nx, model.ny, model.dx, model.dy, radii.tobytes())
    ev = _EVENT_CACHE.get(key)
    if ev is None:
        ev = list(face_events(model, radii))
        _EVENT_CACHE.clear()
        _EVENT_CACHE[key] = ev
    return ev


# --------------------------------------------------------------------------
# Mirroring, FFT, assembly
# --------------------------------------------------------------------------

MIRROR = {"xx": (1, 1), "yy": (1, 1), "zz": (1, 1), "xy": (-1, -1), "xz": (-1, 1), "yz": (1, -1)}


def populate(quadrant, xs, ys):
    """``GreenTensorFftPopulator.PopulateForFft`` (``GreenTensorFftPopulator.cs:221-273``):
    [Nx, Ny, block] -> [2Nx, 2Ny, block] circulant with parity signs; row
    ``Nx`` and column ``Ny`` stay zero."""
    nx, ny, blk = quadrant.shape
    g = np.zeros((2 * nx, 2 * ny, blk), np.complex128)
    g[:nx, :ny] = quadrant
    i = np.arange(1, nx)
    j = np.arange(1, ny)
    g[2 * nx - i[:, None], j[None, :]] = xs * quadrant[1:, 1:]
    g[i[:, None], 2 * ny - j[None, :]] = ys * quadrant[1:, 1:]
    g[2 * nx - i[:, None], 2 * ny - j[None, :]] = (xs * ys) * quadrant[1:, 1:]
    g[2 * nx - i, 0] = xs * quadrant[1:, 0]
    g[0, 2 * ny - j] = ys * quadrant[0, 1:]
    return g


def fft2_forward(g):
    """FFTW ``plan_many_dft`` rank 2, sign -1, unnormalised, over the two
    lateral axes (``Fft/FftW/FftWTransform.cs:218-225``)."""
    return np.fft.fft2(g, axes=(0, 1))


def realspace_tensor(om, n_hankels=10):
    """Real-space quadrant of all six components (before mirroring/FFT):
    dict c -> [Nx, Ny, block]."""
    m = om.model
    hankel = Hankel()
    radii_a, sc_a = compute_scalars(om, n_hankels, asym_transceivers(m), [3], hankel)
    segs_a = segments(radii_a, sc_a)
    qa = integrate_tensor(m, radii_a, segs_a, ["xz", "yz"])
    radii_s, sc_s = compute_scalars(om, n_hankels, symm_transceivers(m), [1, 2, 5], hankel)
    segs_s = segments(radii_s, sc_s)
    qs = integrate_tensor(m, radii_s, segs_s, ["xx", "xy", "yy", "zz"])
    qa.update(qs)
    return qa


def green_tensor(om, n_hankels=10, realspace=None):
    """Spectral AtoA tensor in the reference layout: dict c -> [2Nx, 2Ny, block],
    block = Nz*(Nz+1)/2 packed (xx, xy, yy, zz) or Nz*Nz (xz, yz)."""
    q = realspace if realspace is not None else realspace_tensor(om, n_hankels)
    out = {}
    for c, v in q.items():
        xs, ys = MIRROR[c]
        out[c] = fft2_forward(populate(v, xs, ys))
    return out
