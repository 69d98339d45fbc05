"""CPU: the oracle against the reference's own compiled C code, against the
committed golden vectors, and against closed forms."""
import os

import numpy as np
import pytest

from extreme_gb300.model import OmegaModel, small_model
from oracle import fgmres, green, mt, ref
from oracle import operator as op

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "tiny.npz")


def _tiny():
    from tests.golden.make_golden import tiny_model
    m = tiny_model()
    return m, OmegaModel.build(m, 1.0)


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


def rel(a, b):
    return np.linalg.norm(np.ravel(a) - np.ravel(b)) / np.linalg.norm(np.ravel(b))


# ---------------------------------------------------------------- pins
def test_rho_step_is_float_rounded(gold):
    h = green.Hankel()
    assert h.rho_step() == float(np.float32(10.0 ** float(np.float32(1) / np.float32(40))))
    assert h.rho_step() != 10.0 ** (1.0 / 40)
    assert h.rho_step() == gold["oracle_rho_step"]


def test_plan_matches_golden(gold):
    m, _ = _tiny()
    items = green.anomaly_plan(m.dx, m.dy, m.nx, m.ny, 4)
    np.testing.assert_array_equal(items[0][0], gold["oracle_rho0"])
    np.testing.assert_array_equal(items[0][1], gold["oracle_lambda0"])
    np.testing.assert_array_equal(items[-1][0], gold["oracle_rho_last"])
    # radii cover [min(dx,dy)/2, diagonal] and lambdas run 1/rho_min * step^(130 - i)
    assert items[0][0][0] == min(m.dx, m.dy) / 2
    assert items[0][1][130] == 1.0 / items[0][0][0]


def test_eta_matches_reference_c(gold):
    m, om = _tiny()
    lam = gold["oracle_lambda0"]
    eta, _ = green.layer_eta_exp(om, lam)
    np.testing.assert_array_equal(eta, gold["ref_eta"])


def test_exp_sums_match_reference_c(gold):
    m, om = _tiny()
    lam = gold["oracle_lambda0"]
    eta, _ = green.layer_eta_exp(om, lam)
    tops = m.section.layer_tops()
    for n, (r1, r2, s1, s2) in enumerate(green.asym_transceivers(m)[:9]):
        r = green.corresponding_layer(tops, m.section.thickness, r1 + (r2 - r1) / 2)
        s = green.corresponding_layer(tops, m.section.thickness, s1 + (s2 - s1) / 2)
        t, b = min(r, s), max(r, s)
        mine = green.exp_sums(eta, r, s, t, b, tops[t], tops[b + 1], r1, r2, s1, s2)
        for k in range(6):
            want = gold["ref_exp_sums"][n, k]
            fin = np.isfinite(want)
            np.testing.assert_array_equal(np.isfinite(mine[k]), fin)
            np.testing.assert_allclose(mine[k][fin], want[fin], rtol=1e-13, atol=0)


def test_contraction_matches_reference_c(gold):
    m, _ = _tiny()
    P = 4 * m.nx * m.ny
    G = {c: gold["oracle_G_" + c].reshape(P, -1) for c in ("xx", "xy", "yy", "zz", "xz", "yz")}
    src = gold["contract_src"].reshape(P, 3, m.nz)
    mine = op.contract(G, src, m.nz).reshape(-1)
    assert rel(mine, gold["ref_full_zgemv"]) < 1e-14


def test_threaded_c_contraction_matches_golden(gold):
    """The C restatement timed as the CPU baseline gives the reference's
    FullZgemv golden output too, and agrees with the numpy oracle on a
    ragged random case."""
    from oracle import ccontract
    m, _ = _tiny()
    P = 4 * m.nx * m.ny
    G = {c: gold["oracle_G_" + c].reshape(P, -1) for c in ("xx", "xy", "yy", "zz", "xz", "yz")}
    src = gold["contract_src"].reshape(P, 3, m.nz)
    assert rel(ccontract.contract(G, src, m.nz, 2).reshape(-1), gold["ref_full_zgemv"]) < 1e-14
    rng = np.random.default_rng(5)
    nz, pts = 13, (3, 7)
    s = nz * (nz + 1) // 2
    G = {c: rng.standard_normal(pts + (s,)) + 1j * rng.standard_normal(pts + (s,)) for c in ("xx", "xy", "yy", "zz")}
    for c in ("xz", "yz"):
        G[c] = rng.standard_normal(pts + (nz * nz,)) + 1j * rng.standard_normal(pts + (nz * nz,))
    x = rng.standard_normal(pts + (3, nz)) + 1j * rng.standard_normal(pts + (3, nz))
    assert rel(ccontract.contract(G, x, nz), op.contract(G, x, nz)) < 1e-14


@pytest.mark.skipif(ref.load() is None, reason="oracle/_ref not built (needs the reference tree)")
def test_exp_sums_live_reference_small_model():
    """Live comparison on the 32x32x8 model when the reference C is built here."""
    m = small_model()
    om = OmegaModel.build(m, 0.1)
    rho, lam = green.anomaly_plan(m.dx, m.dy, m.nx, m.ny, 10)[3]
    eta, _ = green.layer_eta_exp(om, lam)
    for k in range(len(om.zeta_bg)):
        np.testing.assert_array_equal(eta[k], ref.calc_eta(lam, green.eta_shift(om.omega, om.zeta_bg[k])))
    tops = m.section.layer_tops()
    for (r1, r2, s1, s2) in green.symm_transceivers(m)[::7]:
        r = green.corresponding_layer(tops, m.section.thickness, r1 + (r2 - r1) / 2)
        s = green.corresponding_layer(tops, m.section.thickness, s1 + (s2 - s1) / 2)
        t, b = min(r, s), max(r, s)
        mine = green.exp_sums(eta, r, s, t, b, tops[t], tops[b + 1], r1, r2, s1, s2)
        for k, name in enumerate(("CalculateT", "CalculateR", "CalculateCTop", "CalculateCBot",
                                  "CalculateDTop", "CalculateDBot")):
            want = ref.exp_sum(name, eta, r, s, t, b, tops[t], tops[b + 1], r1, r2, s1, s2)
            fin = np.isfinite(want)
            np.testing.assert_allclose(mine[k][fin], want[fin], rtol=1e-13)


@pytest.mark.skipif(ref.load() is None, reason="oracle/_ref not built (needs the reference tree)")
def test_hankel_dot_and_zrotg_match_reference_c():
    h = green.Hankel()
    rng = np.random.default_rng(0)
    fk = rng.standard_normal(500) + 1j * rng.standard_normal(500)
    mine = h.convolve(h.h0, fk, 69)
    want = np.array([ref.hankel_dot(h.h0[::-1], fk, i) for i in range(69)])
    np.testing.assert_allclose(mine, want, rtol=1e-12, atol=1e-30)
    for a, b in [(1 + 2j, 3 - 1j), (0j, 2 + 1j), (1e-3 + 0j, 1e3 - 1e3j)]:
        c1, s1 = fgmres.zrotg(a, b)
        c2, s2 = ref.zrotg(a, b)
        assert abs(c1 - c2) < 1e-15 and abs(s1 - s2) < 1e-15


def test_green_tensor_matches_golden(gold):
    _, om = _tiny()
    G = green.green_tensor(om, 4)
    for c, v in G.items():
        assert rel(v, gold["oracle_G_" + c]) < 1e-12, c


def test_apply_and_solve_match_golden(gold):
    m, om = _tiny()
    G = {c: gold["oracle_G_" + c] for c in ("xx", "xy", "yy", "zz", "xz", "yz")}
    x = gold["x"]
    assert rel(op.apply(G, om, x, op.OP_A), gold["oracle_apply_A"]) < 1e-13
    assert rel(op.apply(G, om, x, op.OP_CHI0), gold["oracle_apply_chi0"]) < 1e-13
    A = op.Operator(G, om, op.OP_A)
    b = gold["oracle_apply_chi0"]
    xs, res = fgmres.fgmres_with_gmres(A, 5, 3, 1e-9, 50).solve(b, b.copy())
    assert res.iterations == int(gold["oracle_solve_iterations"])
    assert A.n_applies == int(gold["oracle_solve_applies"])
    assert rel(xs, gold["oracle_solve_x"]) < 1e-10
    assert rel(mt.normal_field(om, "x"), gold["oracle_e0_x"]) < 1e-14


# ---------------------------------------------------------------- physics
def test_green_parity_and_reciprocity(gold):
    """Spectral parity of each component (GreenTensorFftPopulator signs) and
    symmetry of the packed blocks."""
    m, _ = _tiny()
    n0, n1 = 2 * m.nx, 2 * m.ny
    par = {"xx": (1, 1), "yy": (1, 1), "zz": (1, 1), "xy": (-1, -1), "xz": (-1, 1), "yz": (1, -1)}
    for c, (px, py) in par.items():
        g = gold["oracle_G_" + c]
        kx = (-np.arange(n0)) % n0
        ky = (-np.arange(n1)) % n1
        np.testing.assert_allclose(g[kx], px * g, atol=1e-9 * np.abs(g).max())
        np.testing.assert_allclose(g[:, ky], py * g, atol=1e-9 * np.abs(g).max())


def test_zero_contrast_gives_zero_current():
    m, _ = _tiny()
    bg = m.background_indices()
    m.sigma[:] = m.section.sigma[bg][None, None, :]
    om = OmegaModel.build(m, 1.0)
    e0 = mt.normal_field(om, "x")
    js = mt.scattered_current(om, e0)
    assert np.abs(js).max() == 0.0


def test_plane_wave_homogeneous_half_space():
    """E(z) of a homogeneous half-space decays as exp(i k z), k = sqrt(i w mu0 sigma)
    up to the air normalisation; the ratio of E at two depths is exact."""
    from extreme_gb300.model import CartesianModel, Section1D
    sigma = 0.05
    sec = Section1D(0.0, np.array([0.0, 50000.0, 0.0]), np.array([0.0, sigma, sigma]))
    m = CartesianModel(2, 2, 100.0, 100.0, sec, np.array([0.0]), np.array([100.0]), np.full((2, 2, 1), sigma))
    om = OmegaModel.build(m, 0.5)
    e1 = mt.plane_wave_e(om, 1000.0)
    e2 = mt.plane_wave_e(om, 2000.0)
    k = np.sqrt(1j * om.omega * mt.MU0 * om.zeta_bg[1])
    assert abs(e2 / e1 - np.exp(1j * k * 1000.0)) < 1e-9


def test_fgmres_matches_dense_solve():
    rng = np.random.default_rng(5)
    n = 60
    A = np.eye(n) + 0.3 * (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) / np.sqrt(n)
    b = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    solver = fgmres.fgmres_with_gmres(lambda v: A @ v, 8, 4, 1e-12, 100)
    x, res = solver.solve(b, np.zeros(n, complex))
    assert res.converged
    np.testing.assert_allclose(x, np.linalg.solve(A, b), rtol=1e-9, atol=1e-10)
    # classic GMRES, tiny restart count -> non-converged status, not an exception
    g = fgmres.Gmres(lambda v: A @ v, 2, 1e-14, 2)
    _, r2 = g.solve(b, np.zeros(n, complex))
    assert not r2.converged


def test_fgmres_zero_rhs_shortcut():
    g = fgmres.Gmres(lambda v: 2 * v, 4, 1e-10, 3)
    x, r = g.solve(np.zeros(5, complex), np.ones(5, complex))
    assert r.converged and r.iterations == 0


def test_threaded_apply_matches_the_oracle_apply():
    """The CPU baseline's apply (scipy FFTs on all cores, threaded C
    contraction) equals the numpy oracle's apply."""
    from extreme_gb300.model import OmegaModel, scaled_model
    from oracle import cpu_apply, green
    from oracle import operator as op
    m = scaled_model(8, 6, 4, seed=2)
    om = OmegaModel.build(m, 1.0)
    G = green.green_tensor(om, 10)
    x = np.random.default_rng(1).standard_normal(m.nx * m.ny * 3 * m.nz) + 0.5j
    for t in (op.OP_A, op.OP_CHI0):
        want = op.apply(G, om, x, t)
        got = cpu_apply.ThreadedOperator(G, om, t, threads=2)(x)
        assert np.linalg.norm(got - want) / np.linalg.norm(want) < 1e-13


def test_icgs_pass_orthogonalises():
    from oracle import cpu_apply
    rng = np.random.default_rng(4)
    V, _ = np.linalg.qr(rng.standard_normal((200, 6)) + 1j * rng.standard_normal((200, 6)))
    w = rng.standard_normal(200) + 1j * rng.standard_normal(200)
    w0 = w.copy()
    h, nrm = cpu_apply.icgs_pass(V, 3, w)
    np.testing.assert_allclose(h, V[:, :4].conj().T @ w0, rtol=1e-13)
    assert np.abs(V[:, :4].conj().T @ w).max() < 1e-13
    assert abs(nrm - np.linalg.norm(w)) < 1e-13 * nrm
