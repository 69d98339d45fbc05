"""Generates ``tests/golden/tiny.npz``: golden vectors for an 8x6x3 model.

Two sources:

* the reference's own C code (``Native/Native.Matrix/green_scalar.c``,
  ``full_zgemv.c``), compiled from the reference tree by ``oracle/Makefile``
  into ``oracle/_ref/libntv_math_ref.so`` -- vertical wavenumbers, the six
  exponential sums and the block contraction (``ref_*`` keys);
* the oracle restatement of the C# pipeline -- radius plan, spectral Green
  tensor, operator applies, FGMRES solution and plane-wave field
  (``oracle_*`` keys), kept as a regression pin.

Run from the repository root after ``make -C oracle``:

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from extreme_gb300.model import CartesianModel, OmegaModel, Section1D  # noqa: E402
from oracle import fgmres, green, mt, ref  # noqa: E402
from oracle import operator as op  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tiny.npz")


def tiny_model():
    section = Section1D(0.0, np.array([0.0, 500.0, 1500.0, 0.0]),
                        np.array([0.0, 0.01, 0.1, 0.001]))
    depth = np.array([300.0, 500.0, 700.0])
    thick = np.array([200.0, 200.0, 200.0])
    rng = np.random.default_rng(7)
    sigma = 10.0 ** rng.uniform(-2, 0, (8, 6, 3))
    return CartesianModel(8, 6, 400.0, 300.0, section, depth, thick, sigma, name="tiny-8x6x3",
                          frequencies=[1.0]).validate()


def main():
    m = tiny_model()
    om = OmegaModel.build(m, 1.0)
    out = {"model_sigma": m.sigma, "frequency": np.array(1.0)}
    items = green.anomaly_plan(m.dx, m.dy, m.nx, m.ny, 4)
    out["oracle_rho0"] = items[0][0]
    out["oracle_lambda0"] = items[0][1]
    out["oracle_rho_last"] = items[-1][0]
    out["oracle_rho_step"] = np.array(green.Hankel().rho_step())

    lib = ref.load()
    if lib is None:
        raise SystemExit("build oracle/_ref first (make -C oracle)")
    lam = items[0][1]
    eta, ex = green.layer_eta_exp(om, lam)
    out["ref_eta"] = np.stack([ref.calc_eta(lam, green.eta_shift(om.omega, om.zeta_bg[k]))
                               for k in range(len(om.zeta_bg))])
    tops = m.section.layer_tops()
    sums = []
    for (r1, r2, s1, s2) in green.asym_transceivers(m)[:9]:
        r = green.corresponding_layer(tops, m.section.thickness, r1 + (r2 - r1) / 2)
        s = green.corresponding_layer(tops, m.section.thickness, s1 + (s2 - s1) / 2)
        t, b = min(r, s), max(r, s)
        args = (out["ref_eta"], r, s, t, b, tops[t], tops[b + 1], r1, r2, s1, s2)
        sums.append([ref.exp_sum(name, *args) for name in
                     ("CalculateT", "CalculateR", "CalculateCTop", "CalculateCBot", "CalculateDTop",
                      "CalculateDBot")])
    out["ref_exp_sums"] = np.array(sums)

    G = green.green_tensor(om, 4)
    for c, v in G.items():
        out["oracle_G_" + c] = v
    rng = np.random.default_rng(3)
    n = m.nx * m.ny * 3 * m.nz
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    out["x"] = x
    P = 4 * m.nx * m.ny
    Gf = {c: v.reshape(P, -1) for c, v in G.items()}
    src = rng.standard_normal(P * 3 * m.nz) + 1j * rng.standard_normal(P * 3 * m.nz)
    out["contract_src"] = src
    out["ref_full_zgemv"] = ref.full_zgemv(m.nz, Gf["xx"], Gf["xy"], Gf["xz"], Gf["yy"], Gf["yz"], Gf["zz"], src)
    out["oracle_apply_A"] = op.apply(G, om, x, op.OP_A)
    out["oracle_apply_chi0"] = op.apply(G, om, x, op.OP_CHI0)
    A = op.Operator(G, om, op.OP_A)
    b = out["oracle_apply_chi0"]
    solver = fgmres.fgmres_with_gmres(A, 5, 3, 1e-9, 50)
    xs, res = solver.solve(b, b.copy())
    out["oracle_solve_x"] = xs
    out["oracle_solve_iterations"] = np.array(res.iterations)
    out["oracle_solve_applies"] = np.array(A.n_applies)
    out["oracle_e0_x"] = mt.normal_field(om, "x")
    np.savez_compressed(OUT, **out)
    print("wrote", OUT, os.path.getsize(OUT), "bytes; iterations", res.iterations, "applies", A.n_applies)


if __name__ == "__main__":
    main()
