"""Oracle (TEST INFRASTRUCTURE ONLY, see ``oracle/__init__.py``): restarted GMRES / flexible GMRES with a GMRES preconditioner,
numpy complex128, following ``Extreme.Fgmres`` step by step.

* ``GmresSolver.Solve`` (``Extreme.Fgmres/Gmres.cs:77-143``): zero-rhs
  shortcut, user initial guess (one apply for ``r0 = b - A x0``), exact-guess
  check, restart loop with the true residual at restart (``:145-175``);
* ``KrylovSubspaceConstruction`` (``:233-295``): iterative classical
  Gram-Schmidt (re-run while ``2||w|| <= sqrt(sum|h|^2)``, at most 3 passes,
  ``:297-313``), complex Givens rotations (``zrotg``/``zrot``), Arnoldi
  backward error ``|g_{j+1}| / ||b||``;
* ``ConstructCurrentSolution`` (``:187-196``): upper-triangular solve and
  the projection on the (preconditioned) basis;
* ``FinalActions``/``CheckBackwardError`` (``:177-230``): one more apply for
  the true residual unless ``CheckArnoldiOnly``;
* ``FlexibleGmresSolver`` (``FlexibleGmresSolver.cs:24-36``) stores
  ``Z[:, j] = M(V[:, j])``; ``FlexibleGmresWithGmresPreconditioner``
  (``FlexibleGmresWithGmresPreconditioner.cs:105-134``) uses a classic GMRES
  with ``m_in`` vectors, the outer tolerance, one cycle, ``x0 = rhs`` and
  Arnoldi-only checking as ``M``.
"""
import numpy as np

CHECK_ARNOLDI_ONLY = 0
CHECK_WITH_WARNING = 1


def zrotg(a, b):
    """Classic reference ``ZROTG``."""
    if abs(a) == 0.0:
        return 0.0, complex(1.0, 0.0)
    scale = abs(a) + abs(b)
    norm = scale * np.sqrt(abs(a / scale) ** 2 + abs(b / scale) ** 2)
    alpha = a / abs(a)
    return abs(a) / norm, alpha * np.conj(b) / norm


def zrot(x, y, c, s):
    return c * x + s * y, c * y - np.conj(s) * x


def _norm(v):
    return float(np.sqrt(np.vdot(v, v).real))


class Result:
    def __init__(self, converged, arnoldi_be, true_be, iterations):
        self.converged = converged
        self.arnoldi_be = arnoldi_be
        self.true_be = true_be
        self.iterations = iterations


class Gmres:
    """``GmresSolver`` with a right preconditioner ``precond`` (None: the
    classic solver, identity; else the flexible solver)."""

    def __init__(self, apply, m, tol, max_restarts, precond=None,
                 check=CHECK_WITH_WARNING, log=None):
        self.apply = apply
        self.m = m
        self.tol = tol
        self.max_restarts = max_restarts
        self.precond = precond
        self.check = check
        self.log = log

    def solve(self, b, x0):
        m = self.m
        n = b.size
        self.iters = 0
        bn = _norm(b)
        if bn == 0:
            return np.zeros_like(b) if x0 is None else x0.copy(), Result(True, 0, 0, 0)
        result = x0.copy()
        r0 = b - self.apply(result)
        w = r0.copy()
        beta = _norm(w)
        if beta == 0:
            return result, Result(True, 0, 0, 1)
        V = np.zeros((n, m), np.complex128)
        Z = np.zeros((n, m), np.complex128) if self.precond is not None else None
        H = np.zeros((m + 1, m + 1), np.complex128)
        cs = np.zeros(m)
        sn = np.zeros(m, np.complex128)
        it = 0
        while True:
            V[:, 0] = (1 / beta) * w
            H[0, m] = beta
            H[1:, m] = 0
            jh, bea = self._arnoldi(V, Z, H, cs, sn, bn)
            if bea < self.tol:
                be = self._final(jh, V, Z, H, b, result)
                return result, Result(True, bea, be, self.iters)
            it += 1
            if it >= self.max_restarts:
                break
            self._construct(jh, V, Z, H, result)
            r0 = b - self.apply(result.copy())
            w = r0.copy()
            beta = _norm(w)
        be = self._final(m, V, Z, H, b, result)
        return result, Result(False, bea, be, self.iters)

    def _arnoldi(self, V, Z, H, cs, sn, bn):
        m = self.m
        jh = 0
        bea = -1.0
        while True:
            if self.precond is not None:
                Z[:, jh] = self.precond(V[:, jh].copy())
                w = Z[:, jh].copy()
            else:
                w = V[:, jh].copy()
            w = self.apply(w)
            H[:jh + 1, jh] = 0
            northo = 0
            while True:
                northo += 1
                basis = V[:, :jh + 1]
                dots = basis.conj().T @ w
                H[:jh + 1, jh] += dots
                w = w - basis @ dots
                dloo = float(np.sqrt(np.sum(np.abs(dots) ** 2))) ** 2
                dnormw = _norm(w)
                if not (2.0 * dnormw <= np.sqrt(dloo) and northo < 3):
                    break
            H[jh + 1, jh] = dnormw
            if jh < m - 1:
                # at a breakdown (||w|| = 0) the reference divides by zero as
                # well; that column is NaN and never read (bea is then 0)
                with np.errstate(divide="ignore", invalid="ignore"):
                    V[:, jh + 1] = w / dnormw
            for j in range(jh):
                H[j, jh], H[j + 1, jh] = zrot(H[j, jh], H[j + 1, jh], cs[j], sn[j])
            c, s = zrotg(H[jh, jh], H[jh + 1, jh])
            cs[jh], sn[jh] = c, s
            H[jh, m], H[jh + 1, m] = zrot(H[jh, m], H[jh + 1, m], c, s)
            H[jh, jh], H[jh + 1, jh] = zrot(H[jh, jh], H[jh + 1, jh], c, s)
            H[jh + 1, jh] = 0
            bea = abs(H[jh + 1, m]) / bn
            self.iters += 1
            if self.log is not None:
                self.log(self.iters, bea)
            jh += 1
            if not (bea > self.tol and jh < m):
                return jh, bea

    def _construct(self, jh, V, Z, H, result):
        y = H[:jh, self.m].copy()
        for j in range(jh - 1, -1, -1):
            if y[j] != 0:
                y[j] = y[j] / H[j, j]
                y[:j] -= y[j] * H[:j, j]
        basis = Z if Z is not None else V
        corr = basis[:, :jh] @ y
        result[:] = result + corr
        return corr

    def _final(self, jh, V, Z, H, b, result):
        self._construct(jh, V, Z, H, result)
        if self.check == CHECK_ARNOLDI_ONLY:
            return -1.0
        w = b - self.apply(result.copy())
        return _norm(w) / _norm(b)


def fgmres_with_gmres(apply, m_out, m_in, tol, max_restarts, log=None):
    """``FlexibleGmresWithGmresPreconditioner`` around ``apply``; returns a
    solver whose ``solve(b, x0)`` gives (x, Result)."""
    inner = Gmres(apply, m_in, tol, 1, precond=None, check=CHECK_ARNOLDI_ONLY)

    def precond(v):
        z, _ = inner.solve(v, v)
        return z

    return Gmres(apply, m_out, tol, max_restarts, precond=precond,
                 check=CHECK_WITH_WARNING, log=log)
