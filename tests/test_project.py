"""CPU: model/project files and the plain-text exporter.

* ``.xmodel`` / ``.xproj`` written by this package read back identically;
  Applique text fills rows along y and runs along x in single precision
  (``AnomalyLoaderUtils.cs:70-170``); the reader rejects what the reference
  rejects (wrong version, missing sections, short or long lines).
* The reference's own COMMEMI3D2 example deck (a committed fixture) parses.
* The exporter writes .NET ``E``/``F2`` numbers and the reference's file
  names and column heads (``PlainTextExporter.cs``), and its values equal the
  response formulas (impedance via ``egx_mt_responses``, host arithmetic).
"""
import os

import numpy as np
import pytest

from extreme_gb300 import project as pj
from extreme_gb300.export import PlainTextExporter, cs_e, read_table, tipper
from extreme_gb300.forward import LevelResult, MtSolution
from extreme_gb300.model import MU0, freq_to_omega, random_model

# the reference's COMMEMI3D2 example deck (EndUser/ExtremeMt/Examples/COMMEMI3D2),
# committed as a fixture by tests/golden/copy_commemi3d2.py
REFERENCE_DECK = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "commemi3d2")


def test_model_round_trip(tmp_path):
    m = random_model(12, 9, 6, seed=4)
    path = str(tmp_path / "m.xmodel")
    pj.write_model(path, m)
    r = pj.read_model(path)
    assert (r.nx, r.ny, r.nz, r.dx, r.dy) == (m.nx, m.ny, m.nz, m.dx, m.dy)
    np.testing.assert_array_equal(r.sigma, m.sigma)
    np.testing.assert_array_equal(r.layer_depth, m.layer_depth)
    np.testing.assert_array_equal(r.layer_thickness, m.layer_thickness)
    np.testing.assert_array_equal(r.section.thickness, m.section.thickness)
    np.testing.assert_array_equal(r.section.sigma, m.section.sigma)
    assert r.section.zero_air_level == m.section.zero_air_level


def _deck(tmp_path, body, version="2.0"):
    p = tmp_path / "a.xmodel"
    p.write_text('<?xml version="1.0" encoding="utf-8"?>\n<CartesianModel version="%s">%s</CartesianModel>'
                 % (version, body))
    return str(p)


LAT_BG = ('<LateralDimensions nx="4" ny="3" dx="100" dy="50" />'
          '<Background1DSection zeroLevel="0"><Layer thickness="0" sigma="0" />'
          '<Layer thickness="1000" sigma="0.01" /><Layer thickness="0" sigma="0.1" /></Background1DSection>')


def test_applique(tmp_path):
    body = LAT_BG + ('<Anomaly><AnomalyLayer depth="0" thickness="100"><Applique>\n'
                     '2LINES: 1*0.5 3*0.1\n 1lines: 4*2.3E-1\n</Applique></AnomalyLayer></Anomaly>')
    m = pj.read_model(_deck(tmp_path, body))
    want = np.zeros((4, 3))
    want[0, 0:2] = np.float32(0.5)
    want[1:4, 0:2] = np.float32(0.1)
    want[:, 2] = np.float32(0.23)
    np.testing.assert_array_equal(m.sigma[:, :, 0], want)


def test_plain_text_layer_with_fortran_exponents(tmp_path):
    (tmp_path / "l0.dat").write_text("1D-2 2D-2\t3E-2\n4 5 6\n7 8 9\n1 1 1\n")
    body = LAT_BG + ('<Anomaly><AnomalyLayer depth="0" thickness="100">'
                     '<FromFile fileType="plain-text" fileName="l0.dat" /></AnomalyLayer></Anomaly>')
    m = pj.read_model(_deck(tmp_path, body))
    np.testing.assert_array_equal(m.sigma[0, :, 0], [0.01, 0.02, 0.03])
    np.testing.assert_array_equal(m.sigma[3, :, 0], [1, 1, 1])


@pytest.mark.parametrize("case", ["version", "lateral", "background", "short_line", "few_lines", "applique_range"])
def test_reader_rejects(tmp_path, case):
    layer = '<Anomaly><AnomalyLayer depth="0" thickness="100"><FromFile fileType="plain-text" fileName="l.dat" />' \
            '</AnomalyLayer></Anomaly>'
    (tmp_path / "l.dat").write_text("1 1 1\n1 1 1\n1 1 1\n1 1 1\n")
    if case == "version":
        path = _deck(tmp_path, LAT_BG, version="1.0")
    elif case == "lateral":
        path = _deck(tmp_path, LAT_BG.split("/>", 1)[1])
    elif case == "background":
        path = _deck(tmp_path, LAT_BG.split("/>", 1)[0] + "/>")
    elif case == "short_line":
        (tmp_path / "l.dat").write_text("1 1 1\n1 1\n1 1 1\n1 1 1\n")
        path = _deck(tmp_path, LAT_BG + layer)
    elif case == "few_lines":
        (tmp_path / "l.dat").write_text("1 1 1\n1 1 1\n")
        path = _deck(tmp_path, LAT_BG + layer)
    else:
        path = _deck(tmp_path, LAT_BG + '<Anomaly><AnomalyLayer depth="0" thickness="100"><Applique>'
                     '4LINES: 4*1</Applique></AnomalyLayer></Anomaly>')
    with pytest.raises(pj.ModelLoadError):
        pj.read_model(path)


def test_project_round_trip_and_defaults(tmp_path):
    p = pj.Project([0.1, 0.01], [pj.ObservationLevel(0.0, -200.0, 50.0, "surface"), pj.ObservationLevel(100.0)],
                   model_file="m.xmodel", results_path="out",
                   forward=pj.ForwardProjectSettings(7, 12, 30, 5, 1e-9))
    path = str(tmp_path / "p.xproj")
    pj.write_project(path, p)
    r = pj.read_project(path)
    assert r.frequencies == [0.1, 0.01]
    assert r.levels == p.levels
    assert r.forward == p.forward
    assert r.model_path() == str(tmp_path / "m.xmodel") and r.results_dir() == str(tmp_path / "out")
    (tmp_path / "q.xproj").write_text('<ExtremeProject version="0.7.2"><Frequencies><F>1</F></Frequencies>'
                                      '</ExtremeProject>')
    q = pj.read_project(str(tmp_path / "q.xproj"))
    assert q.forward == pj.ForwardProjectSettings(10, 10, 10, 10, 1e-10)
    assert q.levels == [] and q.sites == []


def test_reference_example_deck():
    p = pj.read_project(os.path.join(REFERENCE_DECK, "forward.xproj"))
    m = pj.read_model(p.model_path())
    assert p.frequencies == [0.1, 0.01, 0.001]
    assert len(p.levels) == 4 and {(lv.x_shift, lv.y_shift) for lv in p.levels} == \
        {(-20000.0, -20000.0), (-20000.0, 20000.0), (20000.0, -20000.0), (20000.0, 20000.0)}
    assert p.forward == pj.ForwardProjectSettings(10, 15, 100, 5, 1e-10)
    assert (m.nx, m.ny, m.nz, m.dx, m.dy) == (40, 40, 40, 2000.0, 2000.0)
    assert m.section.zero_air_level == -200000.0 and m.section.n_layers == 5
    assert np.all(m.sigma > 0)
    # every layer file parsed as the reference reads it: line i -> x index i
    first = np.loadtxt(os.path.join(REFERENCE_DECK, "anomaly_layer_0000.dat"))
    np.testing.assert_array_equal(m.sigma[:, :, 0], first)


def test_number_formats():
    assert cs_e(1052.033) == "1.052033E+003"
    assert cs_e(-0.000123) == "-1.230000E-004"
    assert cs_e(0.0) == "0.000000E+000"
    assert cs_e(2.5e-300) == "2.500000E-300"
    assert PlainTextExporter.frequency_to_string(0.1) == "0000000000.1000000000"
    assert PlainTextExporter.responses_file_name(0.001) == "responses_freq0000000000.0010000000"
    assert PlainTextExporter.fields_file_name(12.5) == "fields_freq0000000012.5000000000"


def _fake_solution(m, rng):
    def fields():
        return rng.standard_normal((2, m.nx, m.ny, 3)) + 1j * rng.standard_normal((2, m.nx, m.ny, 3))
    lvs = []
    for z, sx, sy in ((0.0, 0.0, 0.0), (50.0, -1000.0, 250.0)):
        ea, ha = fields(), fields()
        e0, h0 = complex(rng.standard_normal(), 1.0), complex(0.5, rng.standard_normal())
        lv = LevelResult(z, sx, sy, None, None, None, None, None, ea, ha, e0, h0)
        en, hn = lv.normal_fields()
        lv.e = ea + en[:, None, None, :]
        lv.h = ha + hn[:, None, None, :]
        lvs.append(lv)
    return MtSolution(0.25, None, None, [], lvs)


def test_exporter_files(tmp_path):
    rng = np.random.default_rng(5)
    m = random_model(5, 4, 3, seed=2)
    sol = _fake_solution(m, rng)
    f = 0.25
    ex = PlainTextExporter(m, sol, f)
    rp, fp = str(tmp_path / "r"), str(tmp_path / "f")
    ex.export_mt_responses(rp)
    ex.export_raw_fields(fp)
    names, rows = read_table(rp)
    assert names[:4] == ["x", "y", "z", "freq"] and names[4:8] == ["Z_XX_re", "Z_XX_im", "Z_XY_re", "Z_XY_im"]
    assert names[-4:] == ["EW_ZX_re", "EW_ZX_im", "EW_ZY_re", "EW_ZY_im"] and len(names) == 28
    assert rows.shape == (2 * m.nx * m.ny, 28)
    with open(rp) as fh:
        fh.readline()
        first = fh.readline()
    assert first.startswith(" " + "250.00".rjust(10) + " " + "250.00".rjust(10) + " " + "0.00".rjust(10) + " ")
    omega = freq_to_omega(f)
    for li, lv in enumerate(sol.levels):
        blk = rows[li * m.nx * m.ny:(li + 1) * m.nx * m.ny]
        i, j = 3, 2
        s = i * m.ny + j
        r = blk[s]
        assert r[0] == pytest.approx(m.dx * i + m.dx / 2 + lv.shift_x) and r[1] == pytest.approx(m.dy * j + m.dy / 2 + lv.shift_y)
        e1, e2, h1, h2 = lv.e[0, i, j], lv.e[1, i, j], lv.h[0, i, j], lv.h[1, i, j]
        det = h1[0] * h2[1] - h2[0] * h1[1]
        z = np.array([[e1[0] * h2[1] - e2[0] * h1[1], -e1[0] * h2[0] + e2[0] * h1[0]],
                      [e1[1] * h2[1] - e2[1] * h1[1], -e1[1] * h2[0] + e2[1] * h1[0]]]) / det
        zz = z.reshape(-1)
        np.testing.assert_allclose(r[4:12:2], zz.real, rtol=2e-6, atol=1e-300)
        np.testing.assert_allclose(r[5:12:2], zz.imag, rtol=2e-6)
        np.testing.assert_allclose(r[12:16], np.abs(zz) ** 2 / (omega * MU0), rtol=2e-6)
        np.testing.assert_allclose(r[16:20], np.angle(zz), rtol=2e-6, atol=1e-6)
        wx, wy = tipper(h1, h2)
        np.testing.assert_allclose(r[20:24], [wx.real, wx.imag, wy.real, wy.imag], rtol=2e-6, atol=1e-6)
    names, rows = read_table(fp)
    assert len(names) == 4 + 48 and names[4] == "N_polX_Ex_re" and names[28] == "A_polX_Ex_re"
    lv = sol.levels[1]
    r = rows[m.nx * m.ny + 7]
    i, j = divmod(7, m.ny)
    assert r[4] == pytest.approx(lv.e_normal.real, rel=2e-6) and r[11] == 0.0    # N_polX_Hx_im
    assert r[10 + 2] == pytest.approx(lv.h_normal.real, rel=2e-6)                  # N_polX_Hy_re
    np.testing.assert_allclose(r[28:34], np.ravel(np.column_stack([lv.e_anomaly[0, i, j].real,
                                                                   lv.e_anomaly[0, i, j].imag])), rtol=2e-6)
