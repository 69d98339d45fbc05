"""Model and project files (``.xmodel`` / ``.xproj``) and the forward run of a
project: read, solve every frequency on the GPU, export.

Formats as the reference reads them:

* ``.xmodel`` (``Extreme.Cartesian/Model/LoadAndSave/ModelReader.cs:21-174``,
  names in ``ModelSerializer.cs:5-31``): root ``CartesianModel`` of version
  ``2.0``; ``LateralDimensions`` (nx, ny, dx, dy); ``Background1DSection``
  (``zeroLevel``, default 0, and ``Layer`` elements of ``thickness`` and
  ``sigma``, the first and last the half-spaces); ``Anomaly`` with
  ``AnomalyLayer`` elements (``depth``, ``thickness``) whose conductivity
  comes from a plain-text file (``FromFile fileType="plain-text"``, path
  relative to the model file) and/or an ``Applique`` text.
* plain-text anomaly layer (``AnomalyLoaderUtils.cs:40-68``): nx lines of ny
  numbers, separated by blanks or tabs, Fortran ``D`` exponents accepted;
  line i is x index i.
* ``Applique`` (``AnomalyLoaderUtils.cs:70-170``): lines ``<n>LINES: c1*v1
  c2*v2 ...``; each line fills n consecutive y rows, the ``c*v`` runs fill x
  from 0; values are read in single precision.
* ``.xproj`` (``Extreme.Cartesian/Project/ProjectReader.cs:27-128``, names in
  ``ProjectSerializer.cs:5-31``): root ``ExtremeProject``; ``Frequencies/F``;
  ``Observations/Tablets/T`` levels (``z``, ``xShift``, ``yShift``, ``name``);
  ``Observations/Sites/S`` sites (``x``, ``y``, ``z``, ``name``);
  ``Sources/Layers/L``; ``ModelFile``; ``ResultsPath``; ``Settings/Forward``
  (``Extreme.Cartesian/Forward/Project/ForwardSettingsReader.cs:10-21``, whose
  defaults apply to missing entries).

``run_project`` is the loop of ``EndUser/ExtremeMt/ExtremeMtSolverRunner.cs:37-111``:
per frequency, the solve, the level fields and the two plain-text files.
"""
import os
import re
import xml.etree.ElementTree as ET
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

from .model import CartesianModel, Section1D


class ModelLoadError(ValueError):
    """A model or project file the reference would reject."""


def _num(el, name, default=None):
    v = el.get(name)
    if v is None:
        if default is None:
            raise ModelLoadError("missing attribute %r of <%s>" % (name, el.tag))
        return default
    return float(v.strip().replace("D", "E").replace("d", "e"))


def _doubles(line):
    try:
        return [float(t.replace("D", "E")) for t in re.split(r"[ \t]+", line.strip()) if t]
    except ValueError as e:
        raise ModelLoadError(str(e)) from e


def read_plain_text_layer(path, nx, ny):
    """One anomaly layer from a plain-text file: [nx, ny]."""
    with open(path) as f:
        lines = [f.readline() for _ in range(nx)]
    if any(ln == "" for ln in lines):
        raise ModelLoadError("model with illegal Nx value")
    out = np.empty((nx, ny))
    for i, ln in enumerate(lines):
        vals = _doubles(ln)
        if len(vals) != ny:
            raise ModelLoadError("model with illegal Ny value in line %d" % i)
        out[i] = vals
    return out


_APPLIQUE_LINES = re.compile(r"(?P<lines>\d+)LINES:", re.IGNORECASE)
_APPLIQUE_RUN = re.compile(r"\s*(?P<columns>\d+)\*(?P<value>[0-9]*\.?[0-9]+([eE][-+]?[0-9]+)*)", re.IGNORECASE)


def apply_applique(text, layer):
    """Fill ``layer`` [nx, ny] from an Applique text in place."""
    nx, ny = layer.shape
    rows = [s.strip() for s in text.split("\n") if s.strip()]
    prev = 0
    for row in rows:
        m = _APPLIQUE_LINES.search(row)
        if m is None:
            raise ModelLoadError("Applique line without a LINES: count: %r" % row)
        n = int(m.group("lines"))
        runs = [(int(r.group("columns")), float(np.float32(r.group("value")))) for r in _APPLIQUE_RUN.finditer(row)]
        if prev + n > ny:
            raise ModelLoadError("Applique nx is out of range")
        if sum(c for c, _ in runs) > nx:
            raise ModelLoadError("Applique ny is out of range")
        for j in range(prev, prev + n):
            col = 0
            for c, v in runs:
                layer[col:col + c, j] = v
                col += c
        prev += n


def read_model(path) -> CartesianModel:
    """``ModelReader.CartesianModelFromX`` + ``PopulateAnomaly``."""
    root = ET.parse(path).getroot()
    if root.tag != "CartesianModel":
        raise ModelLoadError("not a CartesianModel file")
    if root.get("version") != "2.0":
        raise ModelLoadError("Wrong version")
    lat = root.find("LateralDimensions")
    if lat is None:
        raise ModelLoadError("missing lateral dimensions")
    nx, ny = int(lat.get("nx")), int(lat.get("ny"))
    dx, dy = _num(lat, "dx"), _num(lat, "dy")
    bg = root.find("Background1DSection")
    if bg is None:
        raise ModelLoadError("background layers are not presented")
    zero = _num(bg, "zeroLevel", 0.0)
    layers = bg.findall("Layer")
    section = Section1D(zero, np.array([_num(x, "thickness") for x in layers]),
                        np.array([_num(x, "sigma") for x in layers]))
    depth, thick, sig = [], [], []
    base = os.path.dirname(os.path.abspath(path))
    an = root.find("Anomaly")
    for xl in (an.findall("AnomalyLayer") if an is not None else []):
        depth.append(_num(xl, "depth"))
        thick.append(_num(xl, "thickness"))
        layer = np.zeros((nx, ny))
        ff = xl.find("FromFile")
        if ff is not None and ff.get("fileType") == "plain-text" and ff.get("fileName") is not None:
            layer = read_plain_text_layer(os.path.join(base, ff.get("fileName")), nx, ny)
        ap = xl.find("Applique")
        if ap is not None:
            apply_applique(ap.text or "", layer)
        sig.append(layer)
    sigma = np.stack(sig, axis=-1) if sig else np.zeros((nx, ny, 0))
    name = os.path.splitext(os.path.basename(path))[0]
    m = CartesianModel(nx, ny, dx, dy, section, np.array(depth), np.array(thick), sigma, name=name)
    try:
        return m.validate()
    except (AssertionError, ValueError) as e:
        raise ModelLoadError(str(e)) from e


def _fmt(v):
    return repr(float(v))


def write_model(path, model: CartesianModel, layer_files=True):
    """Model file in the format ``read_model`` reads (``ModelWriter.cs``):
    plain-text layer files beside it (``anomaly_layer_KKKK.dat``)."""
    root = ET.Element("CartesianModel", version="2.0")
    ET.SubElement(root, "LateralDimensions", nx=str(model.nx), ny=str(model.ny), dx=_fmt(model.dx), dy=_fmt(model.dy))
    bg = ET.SubElement(root, "Background1DSection", zeroLevel=_fmt(model.section.zero_air_level))
    for t, s in zip(model.section.thickness, model.section.sigma):
        ET.SubElement(bg, "Layer", thickness=_fmt(t), sigma=_fmt(s))
    an = ET.SubElement(root, "Anomaly")
    base = os.path.dirname(os.path.abspath(path))
    for k in range(model.nz):
        xl = ET.SubElement(an, "AnomalyLayer", depth=_fmt(model.layer_depth[k]), thickness=_fmt(model.layer_thickness[k]))
        fname = "anomaly_layer_%04d.dat" % k
        ET.SubElement(xl, "FromFile", fileType="plain-text", fileName=fname)
        if layer_files:
            with open(os.path.join(base, fname), "w") as f:
                for i in range(model.nx):
                    f.write(" ".join(repr(float(v)) for v in model.sigma[i, :, k]) + " \n")
    ET.ElementTree(root).write(path, encoding="utf-8", xml_declaration=True)


@dataclass
class ObservationLevel:
    z: float
    x_shift: float = 0.0
    y_shift: float = 0.0
    name: str = ""


@dataclass
class ObservationSite:
    x: float
    y: float
    z: float
    name: str = ""


@dataclass
class SourceLayer:
    z: float
    x_shift: int = 0
    y_shift: int = 0


@dataclass
class ForwardProjectSettings:
    """``Settings/Forward``; defaults of ``ForwardSettingsReader.cs:12-19``."""
    inner_buffer_length: int = 10
    outer_buffer_length: int = 10
    max_repeats_number: int = 10
    number_of_hankels: int = 10
    residual: float = 1e-10


@dataclass
class Project:
    frequencies: List[float]
    levels: List[ObservationLevel] = field(default_factory=list)
    sites: List[ObservationSite] = field(default_factory=list)
    sources: List[SourceLayer] = field(default_factory=list)
    model_file: Optional[str] = None
    results_path: Optional[str] = None
    forward: ForwardProjectSettings = field(default_factory=ForwardProjectSettings)
    path: Optional[str] = None

    def model_path(self):
        base = os.path.dirname(os.path.abspath(self.path)) if self.path else ""
        return os.path.join(base, self.model_file)

    def results_dir(self):
        base = os.path.dirname(os.path.abspath(self.path)) if self.path else ""
        return os.path.join(base, self.results_path or "")


def _child_text(el, name):
    c = el.find(name) if el is not None else None
    return c.text.strip() if c is not None and c.text is not None else None


def read_project(path) -> Project:
    """``ProjectReader.FromXDocument`` with the forward settings reader."""
    root = ET.parse(path).getroot()
    if root.tag != "ExtremeProject":
        raise ModelLoadError("No ExtremeProject section in project file")
    fr = root.find("Frequencies")
    freqs = [float(f.text) for f in fr.findall("F")] if fr is not None else []
    obs = root.find("Observations")
    levels, sites, sources = [], [], []
    tab = obs.find("Tablets") if obs is not None else None
    for t in (tab.findall("T") if tab is not None else []):
        levels.append(ObservationLevel(_num(t, "z"), _num(t, "xShift", 0.0), _num(t, "yShift", 0.0),
                                       t.get("name", "")))
    st = obs.find("Sites") if obs is not None else None
    for s in (st.findall("S") if st is not None else []):
        sites.append(ObservationSite(_num(s, "x"), _num(s, "y"), _num(s, "z"), s.get("name", "")))
    src = root.find("Sources")
    sl = src.find("Layers") if src is not None else None
    for s in (sl.findall("L") if sl is not None else []):
        sources.append(SourceLayer(_num(s, "z"), int(_num(s, "xShift", 0.0)), int(_num(s, "yShift", 0.0))))
    fw = root.find("Settings")
    fw = fw.find("Forward") if fw is not None else None
    d = ForwardProjectSettings()

    def get(name, conv, default):
        v = _child_text(fw, name)
        return conv(v) if v else default

    settings = ForwardProjectSettings(get("InnerBufferLength", int, d.inner_buffer_length),
                                      get("OuterBufferLength", int, d.outer_buffer_length),
                                      get("MaxRepeatsNumber", int, d.max_repeats_number),
                                      get("NumberOfHankels", int, d.number_of_hankels),
                                      get("Residual", float, d.residual))
    return Project(freqs, levels, sites, sources, _child_text(root, "ModelFile"), _child_text(root, "ResultsPath"),
                   settings, path)


def write_project(path, project: Project):
    """Project file in the format ``read_project`` reads (``ProjectWriter.cs``)."""
    root = ET.Element("ExtremeProject", version="0.7.2")
    ET.SubElement(root, "ProblemType")
    if project.results_path is not None:
        ET.SubElement(root, "ResultsPath").text = project.results_path
    if project.model_file is not None:
        ET.SubElement(root, "ModelFile").text = project.model_file
    fr = ET.SubElement(root, "Frequencies")
    for f in project.frequencies:
        ET.SubElement(fr, "F").text = repr(float(f))
    obs = ET.SubElement(root, "Observations")
    tab = ET.SubElement(obs, "Tablets")
    for lv in project.levels:
        ET.SubElement(tab, "T", xShift=_fmt(lv.x_shift), yShift=_fmt(lv.y_shift), z=_fmt(lv.z), name=lv.name)
    st = ET.SubElement(root, "Settings")
    fw = ET.SubElement(st, "Forward")
    s = project.forward
    for name, v in (("Residual", s.residual), ("InnerBufferLength", s.inner_buffer_length),
                    ("OuterBufferLength", s.outer_buffer_length), ("MaxRepeatsNumber", s.max_repeats_number),
                    ("NumberOfHankels", s.number_of_hankels)):
        ET.SubElement(fw, name).text = repr(v)
    ET.ElementTree(root).write(path, encoding="utf-8", xml_declaration=True)


def run_project(path, ctx=None, precision=None, mixed=None, log=None):
    """Forward run of a project file: for each frequency the solve of both
    polarisations, the fields at every observation level, and the raw-field
    and MT-response files in the results path (``ExtremeMtSolverRunner.Run``
    and ``Export``). Returns the written file paths."""
    from . import egx
    from .export import PlainTextExporter
    from .forward import ForwardSettings, MixedSettings, Mt3DForwardSolver

    project = read_project(path)
    model = read_model(project.model_path())
    s = project.forward
    settings = ForwardSettings(residual=s.residual, inner_buffer_length=s.inner_buffer_length,
                               outer_buffer_length=s.outer_buffer_length, max_repeats_number=s.max_repeats_number,
                               number_of_hankels=s.number_of_hankels)
    solver = Mt3DForwardSolver(settings, precision=egx.PREC_FP64 if precision is None else precision,
                               mixed=mixed or MixedSettings(), ctx=ctx)
    out_dir = project.results_dir()
    os.makedirs(out_dir, exist_ok=True)
    written = []
    levels = [(lv.z, lv.x_shift, lv.y_shift) for lv in project.levels]
    for f in project.frequencies:
        if log:
            log("frequency %g" % f)
        sol = solver.solve(model, f, levels=levels)
        ex = PlainTextExporter(model, sol, f, names=[lv.name for lv in project.levels])
        fields = os.path.join(out_dir, PlainTextExporter.fields_file_name(f))
        responses = os.path.join(out_dir, PlainTextExporter.responses_file_name(f))
        ex.export_raw_fields(fields)
        ex.export_mt_responses(responses)
        written += [fields, responses]
    return written
