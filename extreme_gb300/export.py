"""Plain-text results in the reference's file format
(``Extreme.Cartesian.Magnetotellurics/Results/PlainTextExporter.cs``).

* file names: ``responses_freq<f>`` / ``fields_freq<f>`` with ``<f>`` the
  frequency as ten integer and ten decimal digits (``:27-34``);
* one line per site of every observation level, x index outer, y inner;
  site coordinates are the cell centres plus the level's shift, ``F2``
  (``AllFieldsUtils.cs:11-34``, ``PlainTextExporter.cs:298-312``);
* numbers in .NET's ``E`` format (six decimals, signed three-digit exponent),
  right-aligned in 14 columns, each followed by a blank (``:314-317``);
* ``export_mt_responses`` (``:238-296``): impedance re/im, apparent
  resistivity, phase (radians unless ``phase_in_degree``; sign reversed with
  ``reverse_phase_sign``), magnetic tipper, electric tipper;
* ``export_raw_fields`` (``:134-236``): normal then anomalous E and H of
  polarisations X and Y, re/im of every component;
* ``export_rho_phase_tipper`` (``:67-100``).

The impedance, apparent resistivity and phase come from ``egx_mt_responses``
(``ResponseFunctionsCalculator.CalculateTensor``); the tippers
(``ResponseFunctionsCalculator.CalculateTipper``, ``:98-117``) are computed
here from the same fields.
"""
import numpy as np

from . import egx
from .model import MU0, freq_to_omega


def cs_e(v):
    """.NET ``double.ToString("E")``: d.ddddddE+ddd."""
    v = float(v)
    if np.isnan(v):
        return "NaN"
    if np.isinf(v):
        return "Infinity" if v > 0 else "-Infinity"
    mant, exp = ("%.6E" % v).split("E")
    e = int(exp)
    return "%sE%s%03d" % (mant, "+" if e >= 0 else "-", abs(e))


def _pad(s, n=14):
    return str(s).rjust(n)


def tipper(h1, h2):
    """W_zx, W_zy from the fields of the two polarisations ([..., 3] each)."""
    det = h1[..., 0] * h2[..., 1] - h2[..., 0] * h1[..., 1]
    hi11, hi12 = h2[..., 1] / det, -h2[..., 0] / det
    hi21, hi22 = -h1[..., 1] / det, h1[..., 0] / det
    return h1[..., 2] * hi11 + h2[..., 2] * hi21, h1[..., 2] * hi12 + h2[..., 2] * hi22


class PlainTextExporter:
    def __init__(self, model, solution, frequency, names=None, export_names=False, phase_in_degree=False,
                 reverse_phase_sign=False):
        self.model = model
        self.levels = solution.levels
        self.frequency = frequency
        self.names = names or [""] * len(self.levels)
        self.export_names = export_names
        self.phase_in_degree = phase_in_degree
        self.reverse_phase_sign = reverse_phase_sign

    @staticmethod
    def frequency_to_string(f):
        return "%021.10f" % f

    @staticmethod
    def responses_file_name(f):
        return "responses_freq" + PlainTextExporter.frequency_to_string(f)

    @staticmethod
    def fields_file_name(f):
        return "fields_freq" + PlainTextExporter.frequency_to_string(f)

    # -- common parts
    def _head(self):
        s = _pad("%name") if self.export_names else "%"
        return s + "%s %s %s %s " % (_pad("x", 10), _pad("y", 10), _pad("z", 10), _pad("freq"))

    def _sites(self):
        """(level index, i, j, x, y, z, name) in the reference's order."""
        m = self.model
        for li, lv in enumerate(self.levels):
            for i in range(m.nx):
                for j in range(m.ny):
                    x = m.dx * i + m.dx / 2 + lv.shift_x
                    y = m.dy * j + m.dy / 2 + lv.shift_y
                    yield li, i, j, x, y, lv.z, self.names[li]

    def _coord(self, x, y, z, name):
        s = (name.rjust(15) + " ") if self.export_names else ""
        return s + " %s %s %s " % (_pad("%.2f" % x, 10), _pad("%.2f" % y, 10), _pad("%.2f" % z, 10)) + \
            _pad(cs_e(self.frequency)) + " "

    def _phase(self, z):
        p = np.angle(z)
        if self.phase_in_degree:
            p = p * (180 / np.pi)
        if self.reverse_phase_sign:
            p = -p
        return p

    def _responses(self, lv):
        omega = freq_to_omega(self.frequency)
        imp, _, _ = egx.mt_responses(lv.e[0], lv.e[1], lv.h[0], lv.h[1], omega)  # [n, 2, 2]
        imp = imp.reshape(-1, 4)
        rho = np.abs(imp) ** 2 / (omega * MU0)
        h1, h2 = lv.h[0].reshape(-1, 3), lv.h[1].reshape(-1, 3)
        e1, e2 = lv.e[0].reshape(-1, 3), lv.e[1].reshape(-1, 3)
        w = np.stack(tipper(h1, h2), -1)
        ew = np.stack(tipper(e1, e2), -1)
        return imp, rho, self._phase(imp), w, ew

    # -- files
    def export_mt_responses(self, path):
        cols = ["Z_XX_re", "Z_XX_im", "Z_XY_re", "Z_XY_im", "Z_YX_re", "Z_YX_im", "Z_YY_re", "Z_YY_im",
                "Rho_XX", "Rho_XY", "Rho_YX", "Rho_YY", "Phs_XX", "Phs_XY", "Phs_YX", "Phs_YY",
                "W_ZX_re", "W_ZX_im", "W_ZY_re", "W_ZY_im", "EW_ZX_re", "EW_ZX_im", "EW_ZY_re", "EW_ZY_im"]
        resp = [self._responses(lv) for lv in self.levels]
        ny = self.model.ny
        with open(path, "w", newline="\n") as f:
            f.write(self._head() + "".join(_pad(c) + " " for c in cols) + "\n")
            for li, i, j, x, y, z, name in self._sites():
                imp, rho, ph, w, ew = resp[li]
                s = i * ny + j
                vals = []
                for c in imp[s]:
                    vals += [c.real, c.imag]
                vals += list(rho[s]) + list(ph[s])
                for c in list(w[s]) + list(ew[s]):
                    vals += [c.real, c.imag]
                f.write(self._coord(x, y, z, name) + "".join(_pad(cs_e(v)) + " " for v in vals) + "\n")

    def export_raw_fields(self, path):
        cols = []
        for kind in ("N", "A"):
            for pol in ("X", "Y"):
                for fld in ("E", "H"):
                    for comp in ("x", "y", "z"):
                        cols += ["%s_pol%s_%s%s_re" % (kind, pol, fld, comp), "%s_pol%s_%s%s_im" % (kind, pol, fld, comp)]
        with open(path, "w", newline="\n") as f:
            f.write(self._head() + "".join(_pad(c) + " " for c in cols) + "\n")
            for li, i, j, x, y, z, name in self._sites():
                lv = self.levels[li]
                en, hn = lv.normal_fields()
                vecs = [en[0], hn[0], en[1], hn[1],
                        lv.e_anomaly[0, i, j], lv.h_anomaly[0, i, j], lv.e_anomaly[1, i, j], lv.h_anomaly[1, i, j]]
                vals = []
                for v in vecs:
                    for c in v:
                        vals += [c.real, c.imag]
                f.write(self._coord(x, y, z, name) + "".join(_pad(cs_e(v)) + " " for v in vals) + "\n")

    def export_rho_phase_tipper(self, path):
        cols = ["Rho_XX", "Rho_XY", "Rho_YX", "Rho_YY", "Phs_XX", "Phs_XY", "Phs_YX", "Phs_YY",
                "W_ZX_RE", "W_ZX_IM", "W_ZY_RE", "W_ZY_IM"]
        resp = [self._responses(lv) for lv in self.levels]
        ny = self.model.ny
        with open(path, "w", newline="\n") as f:
            f.write(self._head() + "".join(_pad(c) + " " for c in cols) + "\n")
            for li, i, j, x, y, z, name in self._sites():
                _, rho, ph, w, _ = resp[li]
                s = i * ny + j
                vals = list(rho[s]) + list(ph[s])
                for c in w[s]:
                    vals += [c.real, c.imag]
                f.write(self._coord(x, y, z, name) + "".join(_pad(cs_e(v)) + " " for v in vals) + "\n")


def read_table(path):
    """Header names and the numeric rows of an exported file."""
    with open(path) as f:
        head = f.readline()
        rows = [list(map(float, ln.split())) for ln in f if ln.strip()]
    names = head.replace("%", " ").split()
    return names, np.array(rows)
