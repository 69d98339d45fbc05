"""Batching form: many independent MT solves (model, frequency) of uneven
mesh sizes on one GPU.

Each solve is the full forward solve of ``Mt3DForwardSolver.solve`` (Green
tensor, both polarisations as one stacked system, fields at the observation
levels). Solves run concurrently on several CUDA streams: one library
context (``egx_create``, its own stream and workspaces) and one host thread
per stream, fed from one queue. The Arnoldi decisions run on the device
(the host reads the state once per outer step), and with ``graphs`` the
inner GMRES cycle of every outer step -- a few hundred small kernels on a
small mesh -- is one CUDA-graph launch (``egx_set_graphs``).

``tune`` is the autotuner: per distinct mesh it times every kernel variant
of the complex64 apply (FFT column tile x contraction kernel,
``egx_tune_apply``) and keeps the fastest for that mesh; then it times a
sample of the batch at each candidate (stream count, graphs on/off) and
keeps the fastest.

Mesh sizes: the register FFT covers 2N in {64, 128, 256, 512}, the Stockham
FFT any other 7-smooth 2N; ``smooth_size`` snaps a drawn size to the nearest
N whose 2N is 7-smooth.
"""
import queue
import threading
import time
from typing import List, Optional, Sequence, Tuple

import numpy as np

from . import egx
from .forward import ForwardSettings, MixedSettings, MtSolution, Mt3DForwardSolver
from .model import CartesianModel, random_model


def is_7smooth(n):
    for p in (2, 3, 5, 7):
        while n % p == 0:
            n //= p
    return n == 1


def smooth_size(n):
    """Nearest N (ties to the smaller) with 2N 7-smooth."""
    for d in range(0, n):
        for c in (n - d, n + d):
            if c > 0 and is_7smooth(2 * c):
                return c
    return n


def batching_models(seed=7, n_models=2, lo=(64, 64, 16), hi=(192, 160, 40)):
    """Seeded models of the batching configuration: meshes drawn uniformly in
    [lo, hi], lateral sizes snapped to 7-smooth 2N, the benchmark generator's
    background and boxes."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n_models):
        nx, ny, nz = (int(rng.integers(a, b + 1)) for a, b in zip(lo, hi))
        out.append(random_model(smooth_size(nx), smooth_size(ny), nz, seed=seed * 100 + k))
    return out


class BatchForwardSolver:
    """Solves ``[(model, frequency), ...]`` on ``streams`` concurrent streams
    of one GPU; results in job order."""

    def __init__(self, settings: Optional[ForwardSettings] = None, precision=egx.PREC_MIXED,
                 mixed: Optional[MixedSettings] = None, streams: int = 4, device: int = 0, graphs: bool = False):
        self.settings = settings or ForwardSettings()
        self.precision = precision
        self.mixed = mixed or MixedSettings()
        self.device = device
        self.streams = streams
        self.graphs = graphs
        self.variants = {}      # mesh (nx, ny, nz) -> (fft_tile, contract_variant) from tune()
        self.apply_times = {}   # mesh -> {(tile, variant): ms per apply}
        self._solvers: List[Mt3DForwardSolver] = []
        self._graphs_set = []

    def _ensure(self, n):
        while len(self._solvers) < n:
            ctx = egx.Context(self.device)
            self._solvers.append(Mt3DForwardSolver(self.settings, precision=self.precision, mixed=self.mixed, ctx=ctx))
            self._graphs_set.append(None)

    def _configure(self, k, graphs):
        if self._graphs_set[k] != graphs:
            self._solvers[k].ctx.set_graphs(graphs)
            self._graphs_set[k] = graphs

    def solve(self, jobs: Sequence[Tuple[CartesianModel, float]], levels=(), streams: Optional[int] = None,
              graphs: Optional[bool] = None) -> List[MtSolution]:
        n = max(1, min(streams or self.streams, len(jobs)))
        self._ensure(n)
        for k in range(n):
            self._configure(k, self.graphs if graphs is None else graphs)
        work = queue.Queue()
        for i, job in enumerate(jobs):
            work.put((i, job))
        results: List[Optional[MtSolution]] = [None] * len(jobs)
        errors = []

        def run(solver):
            while not errors:
                try:
                    i, (model, f) = work.get_nowait()
                except queue.Empty:
                    return
                try:
                    # the tuner's kernel variants for this mesh, else the built-in ones
                    solver.ctx.apply_variant(*self.variants.get((model.nx, model.ny, model.nz), (0, 0)))
                    results[i] = solver.solve(model, f, levels=levels)
                except Exception as e:  # noqa: BLE001 -- re-raised in the caller's thread
                    errors.append(e)
                    return

        threads = [threading.Thread(target=run, args=(self._solvers[k],)) for k in range(n)]
        for th in threads:
            th.start()
        for th in threads:
            th.join()
        if errors:
            raise errors[0]
        return results

    def tune_applies(self, jobs, nrhs=2, reps=5):
        """Per distinct mesh of the jobs: build its Green tensor at the first
        job's frequency, prepare the operator and time every kernel variant
        of the complex64 apply (egx_tune_apply); keeps the fastest per mesh."""
        from .forward import model_zeta
        from .model import freq_to_omega
        self._ensure(1)
        ctx = self._solvers[0].ctx
        for model, f in jobs:
            shape = (model.nx, model.ny, model.nz)
            if shape in self.variants:
                continue
            omega = freq_to_omega(f)
            g = ctx.green_build(model, omega, self.settings.number_of_hankels, egx.PREC_MIXED)
            try:
                zeta, zeta0 = model_zeta(model, omega)
                ctx.op_prepare(g, zeta, zeta0, model.layer_thickness, egx.OP_A)
                tile, var, table = ctx.tune_apply(nrhs=nrhs, reps=reps)
            finally:
                g.free()
            self.variants[shape] = (tile, var)
            self.apply_times[shape] = table
        ctx.apply_variant(0, 0)
        return self.variants

    def tune(self, jobs, candidates=(1, 2, 4, 8), graphs=(False, True), sample=None):
        """The autotuner: kernel variants per mesh (``tune_applies``), then
        ``sample`` jobs (default: as many as the largest stream count) timed
        at every (stream count, graphs) candidate; keeps the fastest and
        returns {(count, graphs): seconds}."""
        self.tune_applies(jobs)
        sample = list(jobs[:sample or max(candidates)])
        self._ensure(max(candidates))
        for g in graphs:  # first-call set-up (workspaces, graph capture) outside the timings
            self.solve(sample[:1], streams=1, graphs=g)
        times = {}
        for g in graphs:
            for c in candidates:
                t = time.perf_counter()
                self.solve(sample, streams=c, graphs=g)
                times[(c, g)] = time.perf_counter() - t
        self.streams, self.graphs = min(times, key=times.get)
        return times

    def close(self):
        for s in self._solvers:
            s.ctx.close()
        self._solvers = []
