"""CPU: the oracle's FGMRES on the failure paths of ``GmresSolver.Solve``
(``Extreme.Fgmres/Gmres.cs:77-143``): the zero right-hand side, an exact
initial guess (``CheckForExactSolution``, ``:104-107,350-356``: converged
after one iteration without a Krylov step) and an Arnoldi breakdown
(``||w|| = 0`` on the identity operator: the next basis column is 0/0 and
is never read, the Givens rotation zeroes the residual, converged after one
step). The GPU tests of the same cases compare against these results.
"""
import numpy as np

from oracle import fgmres


def _counting_identity():
    calls = []

    def apply(v):
        calls.append(1)
        return v.copy()
    return apply, calls


def test_zero_rhs():
    apply, calls = _counting_identity()
    b = np.zeros(10, np.complex128)
    x, r = fgmres.fgmres_with_gmres(apply, 5, 3, 1e-9, 10).solve(b, np.ones(10, np.complex128))
    # converged at once, nothing applied, the result left as the guess was
    assert r.converged and r.iterations == 0 and not calls
    np.testing.assert_array_equal(x, np.ones(10))


def test_exact_initial_guess():
    apply, calls = _counting_identity()
    rng = np.random.default_rng(1)
    b = rng.standard_normal(50) + 1j * rng.standard_normal(50)
    x, r = fgmres.fgmres_with_gmres(apply, 5, 3, 1e-9, 10).solve(b, b.copy())
    assert r.converged and r.iterations == 1 and r.arnoldi_be == 0 and r.true_be == 0
    assert len(calls) == 1
    np.testing.assert_array_equal(x, b)


def test_exact_breakdown_on_the_identity():
    """b = 2 e_k: v0 = e_k exactly, w = A z0 - (v0^H w) v0 = 0 exactly."""
    apply, calls = _counting_identity()
    b = np.zeros(40, np.complex128)
    b[7] = 2.0
    x, r = fgmres.fgmres_with_gmres(apply, 5, 3, 1e-9, 10).solve(b, np.zeros_like(b))
    assert r.converged and r.iterations == 1 and r.arnoldi_be == 0 and r.true_be == 0
    # x0 apply, the inner solve's exact-guess apply, w = A z0, the true residual
    assert len(calls) == 4
    np.testing.assert_array_equal(x, b)


def test_near_breakdown_on_the_identity():
    apply, _ = _counting_identity()
    rng = np.random.default_rng(2)
    b = rng.standard_normal(64) + 1j * rng.standard_normal(64)
    x, r = fgmres.fgmres_with_gmres(apply, 5, 3, 1e-9, 10).solve(b, np.zeros_like(b))
    assert r.converged and r.iterations == 1 and r.true_be < 1e-15
    np.testing.assert_allclose(x, b, rtol=1e-14)
