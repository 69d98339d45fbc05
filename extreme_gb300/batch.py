"""Batching form: many independent MT solves (model, frequency) of uneven
mesh sizes on one GPU.

Each solve is the full forward solve of ``Mt3DForwardSolver.solve`` (Green
tensor, both polarisations as one stacked system, fields at the observation
levels). Solves run concurrently on several CUDA streams: one library
context (``egx_create``, its own stream and workspaces) and one host thread
per stream, fed from one queue, so that the host decisions of one solve's
Arnoldi steps (a device-to-host read per step) and its small kernels overlap
with the other solves' work. A whole solve cannot be one CUDA graph: every
Arnoldi step ends in a host decision (breakdown, convergence, restart).

``tune`` is the stream-count autotuner: it times a sample of the batch at
each candidate count and keeps the fastest.

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
                 mixed: Optional[MixedSettings] = None, streams: int = 4, device: int = 0):
        self.settings = settings or ForwardSettings()
        self.precision = precision
        self.mixed = mixed or MixedSettings()
        self.device = device
        self.streams = streams
        self._solvers: List[Mt3DForwardSolver] = []

    def _ensure(self, n):
        while len(self._solvers) < n:
            ctx = egx.Context(self.device)
            self._solvers.append(Mt3DForwardSolver(self.settings, precision=self.precision, mixed=self.mixed, ctx=ctx))

    def solve(self, jobs: Sequence[Tuple[CartesianModel, float]], levels=(), streams: Optional[int] = None) \
            -> List[MtSolution]:
        n = max(1, min(streams or self.streams, len(jobs)))
        self._ensure(n)
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

    def tune(self, jobs, candidates=(1, 2, 4, 8), sample=None):
        """Stream-count autotuner: time ``sample`` jobs (default: as many as
        the largest candidate) at each count, keep the fastest; returns
        {count: seconds} and sets ``self.streams``."""
        sample = list(jobs[:sample or max(candidates)])
        self._ensure(max(candidates))
        self.solve(sample[:1], streams=1)  # first-call set-up outside the timings
        times = {}
        for c in candidates:
            t = time.perf_counter()
            self.solve(sample, streams=c)
            times[c] = time.perf_counter() - t
        self.streams = min(times, key=times.get)
        return times

    def close(self):
        for s in self._solvers:
            s.ctx.close()
        self._solvers = []
