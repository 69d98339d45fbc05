"""CPU: known-answer tests of the ndec-40 Hankel filter (431 taps, the table
the Green tensor uses; HankelCoefficients.cs:37-118) against closed-form
transforms. With the reference's convention (green_scalar.c:43-55 and the
division by rho in the scalar sums) the filter gives
    int_0^inf f(lam) J_n(lam rho) d lam  ~  (1/rho) sum_j rev(h_n)[j] f(lam_{i+j})
on the lambdas of a rho plan (ScalarPlan.CalculateLambdasForLog10). The
pairs (a > 0, r = sqrt(a^2 + rho^2)):
    J0: e^{-a lam} -> 1/r,        lam e^{-a lam} -> a/r^3,
    J1: e^{-a lam} -> (r - a)/(rho r),   lam e^{-a lam} -> rho/r^3.
Bound: 2e-5 of the transform's largest value over rho in [10 m, 20 km]
(measured 1e-7 .. 9e-6)."""
import numpy as np
import pytest

from oracle import green

PAIRS = [
    ("h0", lambda lam, a: np.exp(-a * lam), lambda rho, a, r: 1 / r),
    ("h0", lambda lam, a: lam * np.exp(-a * lam), lambda rho, a, r: a / r ** 3),
    ("h1", lambda lam, a: np.exp(-a * lam), lambda rho, a, r: (r - a) / (rho * r)),
    ("h1", lambda lam, a: lam * np.exp(-a * lam), lambda rho, a, r: rho / r ** 3),
]


@pytest.mark.parametrize("a", [50.0, 300.0, 2000.0])
@pytest.mark.parametrize("pair", range(len(PAIRS)))
def test_filter_matches_closed_form(a, pair):
    H = green.Hankel()
    rho = green.rho_from_min(10.0, 2e4, H.rho_step())
    lam = green.lambdas_for(H, rho)
    which, f, exact = PAIRS[pair]
    got = H.convolve(getattr(H, which), f(lam, a), rho.size) / rho
    want = exact(rho, a, np.sqrt(a * a + rho * rho))
    assert np.max(np.abs(got - want)) <= 2e-5 * np.max(np.abs(want))
