"""Learned flexible preconditioner: data, training and evaluation around the
library's network (``egx_net_*``).

* ``collect_pairs`` -- (residual, GMRES-preconditioner correction) pairs that
  the solver itself generates: the residuals v are orthonormal Arnoldi
  vectors of the operator A on the right-hand sides chi0 of both
  polarisations (the vectors the outer FGMRES hands its preconditioner), the
  targets t = M(v) - v with M the reference's inner preconditioner -- one
  GMRES(m_in) cycle from x0 = v (``FlexibleGmresWithGmresPreconditioner.cs:35-57``)
  -- all through the library on the device.
* ``train`` -- Adam on the GPU through ``egx_net_loss_grad`` /
  ``egx_net_adam`` (BF16 tensor-core forward and backward kernels), each
  batch drawn across solves with their own conductivity channels.
* ``evaluate`` -- held-out solves of the mixed form with the GMRES
  preconditioner (the reference's method), without a preconditioner, and with
  the network as the flexible preconditioner (GMRES as fallback, the FP64
  residual as judge): iterations, operator applies, fallbacks, wall time.

torch holds the device buffers (vectors of the pairs); it is plumbing.
"""
import time
from dataclasses import dataclass, field
from typing import List

import numpy as np

from . import egx
from .forward import ForwardSettings, MixedSettings, Mt3DForwardSolver, model_zeta
from .model import MU0, CartesianModel, freq_to_omega


def log_conductivity(model: CartesianModel, frequency: float):
    """The network's conductivity channel: log10(omega mu0 sigma dx dy)."""
    omega = freq_to_omega(frequency)
    return np.log10(omega * MU0 * np.maximum(model.sigma, 1e-12) * model.dx * model.dy).astype(np.float32)


@dataclass
class PairSet:
    """Pairs of one (model, frequency) on the device: v [k, N], t = M(v) - v
    [k, N] (complex64), and the conductivity channel [nx, ny, nz]."""
    v: object
    t: object
    logsig: np.ndarray


def collect_pairs(ctx: egx.Context, model: CartesianModel, frequency: float, n_vectors=4, m_in=10, tol=1e-7,
                  pols=(0, 1)) -> PairSet:
    """n_vectors Arnoldi vectors per polarisation in ``pols`` and their
    GMRES(m_in) preconditioner outputs."""
    import torch
    omega = freq_to_omega(frequency)
    zeta, zeta0 = model_zeta(model, omega)
    e0 = egx.normal_field(model, omega)
    g = ctx.green_build(model, omega, 10, egx.PREC_FP64)
    dev = torch.device("cuda", torch.cuda.current_device())
    try:
        rhs = []
        ctx.op_prepare(g, zeta, zeta0, model.layer_thickness, egx.OP_CHI0)
        for pol in pols:
            js = np.zeros((model.nx, model.ny, 3, model.nz), complex)
            js[:, :, pol, :] = (zeta - zeta0[None, None, :]) * e0[None, None, :]
            rhs.append(torch.tensor(ctx.op_apply(js.reshape(-1)), device=dev))
        ctx.op_prepare(g, zeta, zeta0, model.layer_thickness, egx.OP_A)

        def A(x):
            x = x.contiguous()
            y = torch.empty_like(x)
            torch.cuda.synchronize()
            ctx.op_apply_dev(x.data_ptr(), y.data_ptr())
            return y

        vs, ts = [], []
        for b in rhs:
            V = [b / torch.linalg.norm(b)]
            for j in range(n_vectors):
                v = V[-1]
                z = v.clone()
                torch.cuda.synchronize()
                # the inner preconditioner: one GMRES(m_in) cycle from x0 = v
                ctx.fgmres_solve_dev(v.data_ptr(), z.data_ptr(), m_out=m_in, m_in=1, tol=tol, max_restarts=1,
                                     precond=egx.PRECOND_NONE, check_true=False)
                vs.append(v.to(torch.complex64))
                ts.append((z - v).to(torch.complex64))
                if j == n_vectors - 1:
                    break
                w = A(v)
                for u in V:
                    w = w - torch.vdot(u, w) * u
                V.append(w / torch.linalg.norm(w))
        return PairSet(torch.stack(vs), torch.stack(ts), log_conductivity(model, frequency))
    finally:
        g.free()


@dataclass
class TrainLog:
    losses: List[float] = field(default_factory=list)
    seconds: float = 0.0


def train(net: egx.SpectralNet, sets: List[PairSet], steps=500, batch=8, lr=1e-3, seed=0) -> TrainLog:
    """Adam on random batches of pairs drawn across the sets; every sample
    carries its own set's conductivity channel."""
    import torch
    rng = np.random.default_rng(seed)
    log = TrainLog()
    t0 = time.perf_counter()
    index = [(i, j) for i, s in enumerate(sets) for j in range(s.v.shape[0])]
    for step in range(steps):
        pick = [index[k] for k in rng.choice(len(index), min(batch, len(index)), replace=False)]
        v = torch.stack([sets[i].v[j] for i, j in pick]).contiguous()
        t = torch.stack([sets[i].t[j] for i, j in pick]).contiguous()
        net.set_model(np.stack([sets[i].logsig for i, _ in pick]))
        torch.cuda.synchronize()
        log.losses.append(net.loss_grad_dev(v.data_ptr(), t.data_ptr(), v.shape[0]))
        net.adam(lr)
    torch.cuda.synchronize()
    log.seconds = time.perf_counter() - t0
    return log


@dataclass
class EvalRow:
    frequency: float
    method: str
    iterations: List[int]
    applies: List[int]
    true_be: List[float]
    seconds: float
    learned_uses: int = 0
    fallbacks: int = 0


def evaluate(ctx: egx.Context, net: egx.SpectralNet, model: CartesianModel, frequency: float,
             mixed: MixedSettings = None) -> List[EvalRow]:
    """The three inner preconditioners on one held-out (model, frequency);
    the Green tensor is built once and shared."""
    import torch
    mixed = mixed or MixedSettings(tol=1e-6)
    solver = Mt3DForwardSolver(ForwardSettings(), precision=egx.PREC_MIXED, mixed=mixed, ctx=ctx)
    g = solver.calculate_green_tensor(model, frequency)
    rows = []
    try:
        for method in ("gmres", "none", "learned"):
            if method == "learned":
                net.set_model(log_conductivity(model, frequency))
                ctx.set_learned(net)
            elif method == "none":
                ctx.set_precond(egx.PRECOND_NONE)
            else:
                ctx.set_learned(None)
            u0, f0 = ctx.learned_stats()
            torch.cuda.synchronize()
            t = time.perf_counter()
            sol = solver.solve(model, frequency, green=g)
            torch.cuda.synchronize()
            dt = time.perf_counter() - t
            u1, f1 = ctx.learned_stats()
            rows.append(EvalRow(frequency, method, [r["iterations"] for r in sol.results],
                                [r["n_applies"] for r in sol.results], [r["true_be"] for r in sol.results], dt,
                                u1 - u0, f1 - f0))
    finally:
        ctx.set_learned(None)
        g.free()
    return rows


def mean_loss(net: egx.SpectralNet, sets: List[PairSet], batch=8) -> float:
    """The loss over every pair of the sets (no parameter update)."""
    import torch
    out = []
    for s in sets:
        net.set_model(s.logsig)
        for i in range(0, s.v.shape[0], batch):
            v = s.v[i:i + batch].contiguous()
            t = s.t[i:i + batch].contiguous()
            torch.cuda.synchronize()
            out.append(net.loss_grad_dev(v.data_ptr(), t.data_ptr(), v.shape[0]))
    return float(np.mean(out))


def main(argv=None):
    """Train on pairs from seeded random models at log-spaced frequencies,
    evaluate on held-out seeds; one JSON line per training chunk and per
    (model, frequency, method)."""
    import argparse
    import json
    from .model import scaled_model
    ap = argparse.ArgumentParser(description=main.__doc__)
    ap.add_argument("--mesh", type=int, nargs=3, default=[128, 128, 32])
    ap.add_argument("--train-models", type=int, default=500)
    ap.add_argument("--train-freqs", type=int, default=4, help="frequencies per training model, 1e-3..10 Hz")
    ap.add_argument("--vectors", type=int, default=1, help="Arnoldi vectors per solve (alternating polarisation)")
    ap.add_argument("--held-out", type=int, nargs="+", default=[31, 32])
    ap.add_argument("--freqs", type=float, nargs="+", default=[0.01, 1.0])
    ap.add_argument("--width", type=int, default=32)
    ap.add_argument("--layers", type=int, default=4)
    ap.add_argument("--steps", type=int, default=3000)
    ap.add_argument("--batch", type=int, default=8)
    ap.add_argument("--lr", type=float, default=1e-3)
    a = ap.parse_args(argv)
    nx, ny, nz = a.mesh
    ctx = egx.Context(0)
    t0 = time.perf_counter()
    rng = np.random.default_rng(2024)
    sets = []
    for s in range(a.train_models):
        m = scaled_model(nx, ny, nz, seed=1000 + s)
        for f in np.logspace(-3, 1, a.train_freqs) * 10 ** rng.uniform(-0.25, 0.25):
            sets.append(collect_pairs(ctx, m, float(f), n_vectors=a.vectors, pols=(len(sets) % 2,)))
    held = [collect_pairs(ctx, scaled_model(nx, ny, nz, seed=s), f, n_vectors=2) for s in a.held_out for f in a.freqs]
    print(json.dumps({"solves": len(sets), "pairs": sum(s.v.shape[0] for s in sets),
                      "held_pairs": sum(s.v.shape[0] for s in held),
                      "seconds": round(time.perf_counter() - t0, 1)}), flush=True)
    net = egx.SpectralNet(ctx, nx, ny, nz, width=a.width, layers=a.layers, seed=0)
    print(json.dumps({"parameters": net.size, "held_loss_untrained": mean_loss(net, held)}), flush=True)
    chunks = 8
    for c in range(chunks):   # cosine schedule in 8 chunks
        lr = a.lr * 0.5 * (1 + np.cos(np.pi * c / chunks))
        log = train(net, sets, steps=a.steps // chunks, batch=a.batch, lr=lr, seed=c)
        print(json.dumps({"chunk": c, "lr": lr, "train_loss": float(np.mean(log.losses[-50:])),
                          "held_loss": mean_loss(net, held), "seconds": round(log.seconds, 2)}), flush=True)
    for s in a.held_out:
        for f in a.freqs:
            for r in evaluate(ctx, net, scaled_model(nx, ny, nz, seed=s), f):
                d = dict(r.__dict__, seed=s)
                print(json.dumps(d), flush=True)
    net.free()
    ctx.close()


if __name__ == "__main__":
    main()
