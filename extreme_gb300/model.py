"""Cartesian MT model description and the seeded synthetic models of the
benchmark configurations.

A model is a 1-D layered background section plus a 3-D anomaly mesh of
``nx x ny x nz`` cells, exactly the data of the reference's ``CartesianModel``
(``Extreme.Cartesian/Model/CartesianModel.cs``): lateral cell sizes ``dx, dy``,
background layers (thickness, conductivity) below a zero-air level, and
anomaly layers (depth, thickness) each with an ``nx x ny`` conductivity grid.

Conventions followed from the reference:

* layer 0 of the background is the upper (air) half-space and the last layer
  the lower half-space; both carry thickness 0
  (``EndUser/ExtremeMt/Examples/COMMEMI3D2/commemi.xmodel:4-10``);
* depth grows downwards, ``GetLayerDepth(k)`` is the top of layer ``k``
  (``Extreme.Cartesian/Model/Omega/OmegaModel.cs:27-38``);
* ``zeta = sigma - i*omega*eps0`` with ``eps0 = 1/(mu0*c^2)``
  (``Extreme.Cartesian/Model/Omega/OmegaModelUtils.cs:52-83``);
* every anomaly layer must lie inside one background layer
  (``Extreme.Cartesian/Model/ModelUtils.cs:160-185``).

Depths and thicknesses are C# ``decimal`` in the reference. Here they are
doubles built from whole centimetres so that sums and comparisons are exact.
"""
from dataclasses import dataclass, field
from typing import List

import numpy as np

MU0 = 4.0 * np.pi * 1.0e-7
EPS0 = 1.0 / (MU0 * 299792458.0 * 299792458.0)


def freq_to_omega(f):
    return 2.0 * np.pi * f


@dataclass
class Section1D:
    """Background layers. ``thickness[0]`` and ``thickness[-1]`` are 0 (the
    two half-spaces); ``sigma`` in S/m."""
    zero_air_level: float
    thickness: np.ndarray
    sigma: np.ndarray

    @property
    def n_layers(self):
        return len(self.thickness)

    def layer_tops(self):
        """Top depth of every layer (``OmegaModel.GetLayerDepth``)."""
        d = np.empty(self.n_layers)
        d[0] = self.zero_air_level
        for k in range(self.n_layers - 1):
            d[k + 1] = d[k] + self.thickness[k]
        return d

    def zeta(self, omega):
        return self.sigma.astype(np.complex128) - 1j * omega * EPS0


@dataclass
class CartesianModel:
    nx: int
    ny: int
    dx: float
    dy: float
    section: Section1D
    layer_depth: np.ndarray      # [nz] top of each anomaly layer
    layer_thickness: np.ndarray  # [nz]
    sigma: np.ndarray            # [nx, ny, nz] anomaly conductivity, S/m
    name: str = ""
    frequencies: List[float] = field(default_factory=list)

    @property
    def nz(self):
        return len(self.layer_depth)

    def background_index(self, k):
        """Background layer that contains anomaly layer ``k``
        (``ModelUtils.FindCorrespondingBackgroundLayerIndex``,
        ``Extreme.Cartesian/Model/ModelUtils.cs:27-50``). The reference sums in
        C# decimal; integer micrometres keep the sums exact here."""
        def um(v):
            return int(round(float(v) * 1e6))
        start = um(self.layer_depth[k])
        end = start + um(self.layer_thickness[k])
        ss = um(self.section.zero_air_level)
        for i in range(self.section.n_layers):
            es = ss + um(self.section.thickness[i])
            if start >= ss and end <= es:
                return i
            ss = es
        raise ValueError("anomaly layer %d is not inside one background layer" % k)

    def background_indices(self):
        return np.array([self.background_index(k) for k in range(self.nz)], dtype=np.int32)

    def validate(self):
        assert self.sigma.shape == (self.nx, self.ny, self.nz)
        self.background_indices()
        assert self.section.thickness[0] == 0 and self.section.thickness[-1] == 0
        return self


def _cm(x):
    """Round a length in metres to whole centimetres."""
    return float(np.round(np.asarray(x) * 100.0) / 100.0)


def small_model():
    """3-layer background (100 Ohm.m 2 km / 10 Ohm.m 8 km / 1000 Ohm.m
    half-space) under air, one 1 Ohm.m cube (2x2 cells, 1-3 km deep) centred
    in a 32x32x8 mesh of 1 km cells and 250 m layers; f = 0.1 Hz."""
    nx = ny = 32
    nz = 8
    section = Section1D(0.0,
                        np.array([0.0, 2000.0, 8000.0, 0.0]),
                        np.array([0.0, 1.0 / 100.0, 1.0 / 10.0, 1.0 / 1000.0]))
    depth = 1000.0 + 250.0 * np.arange(nz)
    thick = np.full(nz, 250.0)
    m = CartesianModel(nx, ny, 1000.0, 1000.0, section, depth, thick,
                       np.zeros((nx, ny, nz)), name="small-32x32x8", frequencies=[0.1])
    bg = m.background_indices()
    m.sigma[:] = section.sigma[bg][None, None, :]
    m.sigma[15:17, 15:17, :] = 1.0
    return m.validate()


def random_model(nx, ny, nz, seed, n_boxes=20, dxy=500.0, dz0=100.0, growth=1.1,
                 frequencies=None, name=None):
    """Seeded generator of the medium/precision configurations: 5 background
    layers with log10(rho) ~ U[0, 3] and thickness ~ U[0.5, 5] km over a
    half-space, interfaces inside the anomaly snapped to anomaly-layer
    boundaries; anomaly layers ``dz_k = dz0 * growth^k`` from the surface;
    ``n_boxes`` axis-aligned boxes with log10(rho) ~ U[-0.5, 3]."""
    rng = np.random.default_rng(seed)
    thick = np.array([_cm(dz0 * growth ** k) for k in range(nz)])
    depth = np.concatenate([[0.0], np.cumsum(thick)[:-1]])
    depth = np.array([_cm(d) for d in depth])
    bottom = _cm(depth[-1] + thick[-1])
    bounds = np.concatenate([depth, [bottom]])

    n_bg = 5
    bg_rho = 10.0 ** rng.uniform(0.0, 3.0, n_bg + 1)
    bg_th = rng.uniform(500.0, 5000.0, n_bg)
    interfaces = np.cumsum(bg_th)
    snapped = []
    for d in interfaces:
        if d < bottom:
            d = bounds[np.argmin(np.abs(bounds - d))]
        d = _cm(d)
        if d <= (snapped[-1] if snapped else 0.0):
            continue
        snapped.append(d)
    if snapped[-1] < bottom:
        snapped.append(_cm(bottom + 10000.0))
    snapped = np.array(snapped)
    thick_bg = np.diff(np.concatenate([[0.0], snapped]))
    n_fin = len(thick_bg)
    section = Section1D(0.0,
                        np.concatenate([[0.0], thick_bg, [0.0]]),
                        np.concatenate([[0.0], 1.0 / bg_rho[:n_fin], [1.0 / bg_rho[-1]]]))
    if frequencies is None:
        frequencies = list(np.logspace(-3, 1, 4))
    m = CartesianModel(nx, ny, dxy, dxy, section, depth, thick, np.zeros((nx, ny, nz)),
                       name=name or "random-%dx%dx%d-s%d" % (nx, ny, nz, seed),
                       frequencies=frequencies)
    bg = m.background_indices()
    m.sigma[:] = section.sigma[bg][None, None, :]
    for _ in range(n_boxes):
        sx = rng.integers(1, max(2, nx // 4) + 1)
        sy = rng.integers(1, max(2, ny // 4) + 1)
        sz = rng.integers(1, max(2, nz // 3) + 1)
        x0 = rng.integers(0, nx - sx + 1)
        y0 = rng.integers(0, ny - sy + 1)
        z0 = rng.integers(0, nz - sz + 1)
        rho = 10.0 ** rng.uniform(-0.5, 3.0)
        m.sigma[x0:x0 + sx, y0:y0 + sy, z0:z0 + sz] = 1.0 / rho
    return m.validate()


def medium_model(seed=1):
    return random_model(128, 128, 32, seed, name="medium-128x128x32")


def precision_model(seed=1):
    return random_model(256, 256, 48, seed, name="precision-256x256x48")


def scaled_model(nx, ny, nz, seed=1):
    """Same generator at an arbitrary mesh size (tests and smaller benches)."""
    return random_model(nx, ny, nz, seed)


@dataclass
class OmegaModel:
    """A model at one angular frequency: the complex conductivities ``zeta``
    of the background layers and the anomaly cells
    (``Extreme.Cartesian/Model/Omega/OmegaModelBuilder.cs:118-158``)."""
    model: CartesianModel
    omega: float
    zeta_bg: np.ndarray      # [L]
    zeta: np.ndarray         # [nx, ny, nz]
    zeta0: np.ndarray        # [nz] background zeta of each anomaly layer
    bg_index: np.ndarray     # [nz]

    @staticmethod
    def build(model: CartesianModel, frequency: float):
        omega = freq_to_omega(frequency)
        zb = model.section.zeta(omega)
        z = model.sigma.astype(np.complex128) - 1j * omega * EPS0
        bg = model.background_indices()
        return OmegaModel(model, omega, zb, z, zb[bg], bg)
