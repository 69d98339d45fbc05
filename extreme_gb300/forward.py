"""Host-side mirror of the reference's forward-solver surface for the IE hot
path, backed by ``libegx.so``.

* :class:`ForwardSettings` -- ``Extreme.Cartesian/Forward/Project/ForwardSettings.cs:8-12``
  (same names and class defaults);
* :class:`Mt3DForwardSolver` -- ``Extreme.Cartesian.Magnetotellurics/Solver/Mt3DForwardSolver.cs:78-129``:
  ``solve(model, frequency)`` computes the anomaly-to-anomaly Green tensor
  (``CalculateGreenTensor``) and then solves polarisation X and Y
  (``SolveForOneSource``: normal field, ``jS``, ``chi0``, FGMRES, ``Es``, ``jQ``),
  then the fields and responses at the observation levels.

Everything numeric runs in the CUDA library: the host only forms the
per-layer plane-wave field (``egx_normal_field``, ``nz`` scalars) and the
complex conductivities ``zeta = sigma - i omega eps0``.
"""
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

from . import egx
from .model import EPS0, CartesianModel, freq_to_omega


@dataclass
class ForwardSettings:
    residual: float = 1e-8
    inner_buffer_length: int = 10
    outer_buffer_length: int = 15
    max_repeats_number: int = 100
    number_of_hankels: int = 10


@dataclass
class MixedSettings:
    """Precision form: inner complex64 FGMRES inside FP64 refinement."""
    tol: float = 1e-6
    max_outer: int = 10
    m_out: int = 30
    m_in: int = 10
    inner_tol: float = 5e-7
    inner_restarts: int = 20
    batch: bool = True        # both polarisations as one stacked system


class TensorCache:
    """Green tensors kept across solves whose geometry and background do not
    change, e.g. the forward solves of an inversion where only the anomaly
    conductivity moves (``Extreme.Cartesian/Forward/TensorCache.cs:8-35``,
    used by ``Mt3DForwardSolver.SolveWithoutGather``,
    ``Mt3DForwardSolver.cs:85-110``): the anomaly-to-anomaly tensor per
    (lateral geometry, anomaly layers, background, frequency, filter length,
    precision). The level tensors are cached inside the context
    (``Context.level_cache``). ``free()`` releases the device memory."""

    def __init__(self):
        self._atoa = {}

    @staticmethod
    def key(model: CartesianModel, frequency, n_hankels, precision):
        sec = model.section
        return (model.nx, model.ny, float(model.dx), float(model.dy), tuple(np.asarray(model.layer_depth, float)),
                tuple(np.asarray(model.layer_thickness, float)), float(sec.zero_air_level),
                tuple(np.asarray(sec.thickness, float)), tuple(np.asarray(sec.sigma, float)), float(frequency),
                int(n_hankels), int(precision))

    def atoa(self, solver, model: CartesianModel, frequency):
        k = self.key(model, frequency, solver.settings.number_of_hankels, solver.precision)
        g = self._atoa.get(k)
        if g is None:
            g = solver.calculate_green_tensor(model, frequency)
            self._atoa[k] = g
        return g

    def __len__(self):
        return len(self._atoa)

    def free(self):
        for g in self._atoa.values():
            g.free()
        self._atoa.clear()


@dataclass
class MtSolution:
    frequency: float
    jq: np.ndarray                      # [2, N]: pol X, pol Y
    chi: Optional[np.ndarray]
    results: List[dict] = field(default_factory=list)
    levels: List["LevelResult"] = field(default_factory=list)


@dataclass
class LevelResult:
    """Fields and responses at the cell centres of one observation level
    (``AllFieldsAtLevel`` / ``AllFieldsAtSite`` and ``ResponseFunctionsCalculator``)."""
    z: float
    shift_x: float
    shift_y: float
    e: np.ndarray          # [2 pols, nx, ny, 3] total E
    h: np.ndarray          # [2 pols, nx, ny, 3] total H
    impedance: np.ndarray  # [nx*ny, 2, 2]
    rho: np.ndarray        # [nx*ny, 2, 2] apparent resistivity, Ohm m
    phase: np.ndarray      # [nx*ny, 2, 2] degrees
    e_anomaly: Optional[np.ndarray] = None  # [2 pols, nx, ny, 3] anomalous E
    h_anomaly: Optional[np.ndarray] = None  # [2 pols, nx, ny, 3] anomalous H
    e_normal: complex = 0j                  # plane-wave E0 at z (pol X: (E0, 0, 0), pol Y: (0, E0, 0))
    h_normal: complex = 0j                  # plane-wave H0 at z (pol X: (0, H0, 0), pol Y: (-H0, 0, 0))

    def normal_fields(self):
        """Normal E and H of both polarisations at every site: [2, 3] each."""
        en = np.array([[self.e_normal, 0, 0], [0, self.e_normal, 0]], complex)
        hn = np.array([[0, self.h_normal, 0], [-self.h_normal, 0, 0]], complex)
        return en, hn


def model_zeta(model: CartesianModel, omega: float):
    """Anomaly and background complex conductivities (OmegaModelUtils.cs:57-83)."""
    zeta = model.sigma.astype(np.complex128) - 1j * omega * EPS0
    bg = model.background_indices()
    zb = model.section.sigma.astype(np.complex128) - 1j * omega * EPS0
    return np.ascontiguousarray(zeta), np.ascontiguousarray(zb[bg])


class Mt3DForwardSolver:
    def __init__(self, settings: ForwardSettings = None, precision=egx.PREC_FP64, mixed: MixedSettings = None,
                 ctx: egx.Context = None, device=0):
        self.settings = settings or ForwardSettings()
        self.precision = precision
        self.mixed = mixed or MixedSettings()
        self.ctx = ctx or egx.Context(device)

    def calculate_green_tensor(self, model: CartesianModel, frequency: float):
        omega = freq_to_omega(frequency)
        return self.ctx.green_build(model, omega, self.settings.number_of_hankels, self.precision)

    def fields_at_level(self, model: CartesianModel, frequency: float, jq, z=0.0, shift_x=0.0, shift_y=0.0):
        """Total fields of both polarisations at the level and the MT
        responses (``Mt3DForwardSolver`` observation path:
        ``AtoOCalculator`` anomalous fields + plane-wave normal fields,
        ``Mt3DForwardSolver.cs:300-337``). The level tensors are built in the
        solver's precision (the mixed form: complex64 lateral FFT)."""
        omega = freq_to_omega(frequency)
        ea, ha = self.ctx.level_fields(model, omega, jq, z=z, shift_x=shift_x, shift_y=shift_y,
                                       n_hankels=self.settings.number_of_hankels, precision=self.precision)
        e_n, h_n = egx.plane_wave(model, omega, z)
        e = ea.copy()
        h = ha.copy()
        e[0, ..., 0] += e_n   # pol X: E = (E0, 0, 0), H = (0, H0, 0)
        h[0, ..., 1] += h_n
        e[1, ..., 1] += e_n   # pol Y: E = (0, E0, 0), H = (-H0, 0, 0)
        h[1, ..., 0] -= h_n
        imp, rho, ph = egx.mt_responses(e[0], e[1], h[0], h[1], omega)
        return LevelResult(z, shift_x, shift_y, e, h, imp, rho, ph, ea, ha, e_n, h_n)

    def solve(self, model: CartesianModel, frequency: float, green=None, want_chi=False,
              levels=(), tensors: Optional[TensorCache] = None) -> MtSolution:
        """Both polarisations to jQ; then, for every level (a depth or a
        (depth, shift_x, shift_y) tuple), fields and responses. With
        ``tensors`` the anomaly-to-anomaly Green tensor comes from (and stays
        in) that cache."""
        omega = freq_to_omega(frequency)
        if green is None and tensors is not None:
            green = tensors.atoa(self, model, frequency)
        own = green is None
        if own:
            green = self.calculate_green_tensor(model, frequency)
        try:
            zeta, zeta0 = model_zeta(model, omega)
            e0 = egx.normal_field(model, omega)
            s = self.settings
            fg = dict(m_out=s.outer_buffer_length, m_in=s.inner_buffer_length, tol=s.residual,
                      max_restarts=s.max_repeats_number)
            mx = self.mixed.__dict__
            jq, chi, res = self.ctx.solve_sources(green, zeta, zeta0, model.layer_thickness,
                                                  np.stack([e0, e0]), [0, 1], precision=self.precision,
                                                  fgmres=fg, mixed=mx, want_chi=want_chi)
        finally:
            if own:
                green.free()
        sol = MtSolution(frequency, jq, chi, res)
        for lv in levels:
            z, sx, sy = (lv, 0.0, 0.0) if np.isscalar(lv) else lv
            sol.levels.append(self.fields_at_level(model, frequency, jq, z, sx, sy))
        return sol
