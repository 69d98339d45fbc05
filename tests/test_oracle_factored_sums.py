"""CPU: the factored form of the Green scalars' four-term exponential sums
that the device kernel computes (each sum = its first term times
(1 - e^{-(r2 - r1) eta_r}) (1 - e^{-(s2 - s1) eta_s})) against the oracle's
term-by-term sums (``oracle.green.exp_sums``, green_scalar.c:86-386), on the
layer geometry of a seeded background and lambdas over the filter's range:
equal to 1e-13 of the leading (largest) term wherever the four-term sum is
finite (the sums cancel, so their own size is no scale), and never infinite
where the four-term sum is finite."""
import numpy as np
import pytest

from oracle import green


def factored(eta, r, s, t, b, dt, db1, r1, r2, s1, s2):
    """(value, leading term) per sum, as the device kernel computes them."""
    er, es, et, eb = eta[r], eta[s], eta[t], eta[b]
    with np.errstate(over="ignore", invalid="ignore"):
        fsr = (1 - np.exp(-(r2 - r1) * er)) * (1 - np.exp(-(s2 - s1) * es))
        first = -2 * db1 * eb + 2 * dt * et
        leads = (np.exp(-r1 * er - s1 * es + 2 * dt * et),
                 np.exp(-2 * db1 * eb + s2 * es + r2 * er),
                 np.exp(-s1 * es + r2 * er),
                 np.exp(-r1 * er + s2 * es),
                 np.exp(first + s2 * es - r1 * er),
                 np.exp(first - s1 * es + r2 * er))
        return [(lead * fsr, lead) for lead in leads]


@pytest.mark.parametrize("omega", [2 * np.pi * 1e-3, 2 * np.pi * 1.0, 2 * np.pi * 100.0])
def test_factored_sums_equal_four_term_sums(omega):
    rng = np.random.default_rng(int(omega * 1000) % 2**31)
    mu0 = 4e-7 * np.pi
    # background: air, 5 layers, half-space; tops in metres
    thick = np.concatenate([[0.0], rng.uniform(500, 5000, 5), [0.0]])
    sigma = np.concatenate([[0.0], 10.0 ** -rng.uniform(0, 3, 5), [10.0 ** -rng.uniform(0, 3)]])
    tops = np.concatenate([[0.0], np.cumsum(thick[:-1])])
    checked = 0
    for lam in 10.0 ** rng.uniform(-7, -1, 40):
        eta = np.sqrt(lam * lam - 1j * omega * mu0 * sigma)
        for _ in range(20):
            # a receiver and a source interval inside finite layers
            r, s = rng.integers(1, 6, 2)
            t, b = min(r, s), max(r, s)
            r1 = tops[r] + rng.uniform(0, thick[r] * 0.9)
            r2 = r1 + rng.uniform(0, tops[r] + thick[r] - r1)
            s1 = tops[s] + rng.uniform(0, thick[s] * 0.9)
            s2 = s1 + rng.uniform(0, tops[s] + thick[s] - s1)
            dt, db1 = tops[t], tops[b + 1]
            want = green.exp_sums(eta, r, s, t, b, dt, db1, r1, r2, s1, s2)
            got = factored(eta, r, s, t, b, dt, db1, r1, r2, s1, s2)
            for w, (g, lead) in zip(want, got):
                if not np.isfinite(w):
                    continue
                assert np.isfinite(g), (w, g)
                # the leading term is the largest of the four: the two forms
                # agree to rounding of the terms' size
                assert abs(g - w) <= 1e-13 * abs(lead) + 1e-300, (w, g, lead)
                checked += 1
    assert checked > 1000
