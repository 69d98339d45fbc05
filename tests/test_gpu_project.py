"""GPU: a project run end to end (``ExtremeMtSolverRunner.Run``): model and
project files written here, read back, both polarisations solved for every
frequency, the fields at two observation levels (one shifted by whole and
half cells) and the two plain-text files per frequency.

The exported numbers must be the solver's own results: the apparent
resistivity and phase of ``Mt3DForwardSolver.solve`` at the same levels, the
normal fields of ``egx_plane_wave`` and the anomalous fields of
``egx_level_fields``; and the fields must agree with the oracle's level
pipeline (to the 7 significant digits that the files carry).
"""
import os

import numpy as np
import pytest

from extreme_gb300 import egx
from extreme_gb300 import project as pj
from extreme_gb300.export import PlainTextExporter, read_table
from extreme_gb300.forward import ForwardSettings, Mt3DForwardSolver
from extreme_gb300.model import OmegaModel, freq_to_omega, random_model
from oracle import atoo, green, mt

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(np.ravel(a) - np.ravel(b)) / np.linalg.norm(np.ravel(b))


def test_project_run(egx_ctx, tmp_path):
    m = random_model(16, 12, 8, seed=11)
    pj.write_model(str(tmp_path / "model.xmodel"), m)
    levels = [pj.ObservationLevel(0.0, 0.0, 0.0, "surface"), pj.ObservationLevel(0.0, -1250.0, 3000.0, "shifted")]
    freqs = [0.1, 3.0]
    proj = pj.Project(freqs, levels, model_file="model.xmodel", results_path="results",
                      forward=pj.ForwardProjectSettings(10, 20, 100, 10, 1e-9))
    path = str(tmp_path / "forward.xproj")
    pj.write_project(path, proj)
    files = pj.run_project(path, ctx=egx_ctx)
    assert [os.path.basename(f) for f in files] == [
        PlainTextExporter.fields_file_name(freqs[0]), PlainTextExporter.responses_file_name(freqs[0]),
        PlainTextExporter.fields_file_name(freqs[1]), PlainTextExporter.responses_file_name(freqs[1])]

    solver = Mt3DForwardSolver(ForwardSettings(residual=1e-9, outer_buffer_length=20), ctx=egx_ctx)
    n_site = m.nx * m.ny
    for k, f in enumerate(freqs):
        sol = solver.solve(m, f, levels=[(lv.z, lv.x_shift, lv.y_shift) for lv in levels])
        names, resp = read_table(files[2 * k + 1])
        _, flds = read_table(files[2 * k])
        assert resp.shape == (2 * n_site, 28) and flds.shape == (2 * n_site, 52)
        for li, lv in enumerate(sol.levels):
            r = resp[li * n_site:(li + 1) * n_site]
            rho, ph = lv.rho.reshape(-1, 4), np.deg2rad(lv.phase.reshape(-1, 4))
            np.testing.assert_allclose(r[:, 12:16], rho, rtol=1e-5)
            np.testing.assert_allclose(r[:, 16:20], ph, rtol=1e-5, atol=1e-5)
            fl = flds[li * n_site:(li + 1) * n_site]
            e_n, h_n = egx.plane_wave(m, freq_to_omega(f), lv.z)
            np.testing.assert_allclose(fl[:, 4], e_n.real, rtol=1e-6)
            np.testing.assert_allclose(fl[:, 12], h_n.real, rtol=1e-6)      # N_polX_Hy_re
            ea = fl[:, 28:34:2] + 1j * fl[:, 29:34:2]                        # A_polX_E
            assert rel(ea, lv.e_anomaly[0].reshape(-1, 3)) < 1e-5

    # the shifted level against the oracle's level pipeline at the first frequency
    om = OmegaModel.build(m, freqs[0])
    G = green.green_tensor(om, 10)
    outs = {p: mt.solve_polarization(om, G, "xy"[p], m_out=20, m_in=10, tol=1e-9) for p in (0, 1)}
    lvl = atoo.Level(levels[1].z, levels[1].x_shift, levels[1].y_shift)
    want = atoo.level_responses(om, lvl, outs[0].jq, outs[1].jq)
    _, resp = read_table(files[1])
    r = resp[n_site:]
    rho_w = want["rho"].reshape(-1, 4)
    # the files carry 7 significant digits
    for c in (1, 2):   # xy, yx
        assert rel(r[:, 12 + c], rho_w[:, c]) < 2e-6
