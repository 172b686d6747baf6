"""Reader and writer of the XMI-MSIM file formats (no libxml2 dependency).

* ``.xmsi`` input files (root ``xmimsim`` or ``xmimsim-input``), element
  grammar of xml/xmimsim-1.0.dtd; reading follows src/xmi_xml.c:1286
  (zero weight fractions dropped, elements sorted by atomic number; the
  library normalises the fractions of every layer in xmi_input_C2F).
* ``.xmso`` result files (root ``xmimsim-results``): convolved and
  unconvolved spectra per interaction order, brute-force and
  variance-reduction line histories, and the embedded input
  (src/xmi_xml.c:1638 writer, :2033 reader).
"""
from __future__ import annotations

import xml.etree.ElementTree as ET
from pathlib import Path

import numpy as np

from .simulation import ContinuousPoint, DiscreteLine, InputSpec, Layer

DETECTOR_TYPES = {"SiLi": 0, "Ge": 1, "Si_SDD": 2}
DIST_TYPES = {"monochromatic": 0, "gaussian": 1, "lorentzian": 2}
ELEMENT_SYMBOLS = (
    "H He Li Be B C N O F Ne Na Mg Al Si P S Cl Ar K Ca Sc Ti V Cr Mn Fe Co Ni Cu Zn Ga Ge As Se Br Kr Rb Sr Y Zr "
    "Nb Mo Tc Ru Rh Pd Ag Cd In Sn Sb Te I Xe Cs Ba La Ce Pr Nd Pm Sm Eu Gd Tb Dy Ho Er Tm Yb Lu Hf Ta W Re Os Ir "
    "Pt Au Hg Tl Pb Bi Po At Rn Fr Ra Ac Th Pa U Np Pu").split()


def _f(node, tag, default=None, cast=float):
    e = node.find(tag)
    if e is None or e.text is None:
        if default is None:
            raise ValueError(f"missing <{tag}> in <{node.tag}>")
        return default
    return cast(e.text.strip())


def _xyz(node, tag):
    e = node.find(tag)
    return (_f(e, "x"), _f(e, "y"), _f(e, "z"))


def _layer(node) -> Layer:
    zw = []
    for el in node.findall("element"):
        z = _f(el, "atomic_number", cast=int)
        w = _f(el, "weight_fraction")
        if abs(w) < 1e-20:
            continue
        zw.append((z, w))
    zw.sort()
    return Layer([z for z, _ in zw], [w for _, w in zw], _f(node, "density"), _f(node, "thickness"))


def parse_input(root) -> InputSpec:
    g = root.find("general")
    comp = root.find("composition")
    geo = root.find("geometry")
    exc = root.find("excitation")
    absb = root.find("absorbers")
    det = root.find("detector")
    layers = [_layer(l) for l in comp.findall("layer")]
    discrete = []
    for d in exc.findall("discrete"):
        sp = d.find("scale_parameter")
        dist = DIST_TYPES.get(sp.get("distribution_type", "monochromatic"), 0) if sp is not None else 0
        discrete.append(DiscreteLine(_f(d, "energy"), _f(d, "horizontal_intensity"), _f(d, "vertical_intensity"),
                                     _f(d, "sigma_x", 0.0), _f(d, "sigma_xp", 0.0), _f(d, "sigma_y", 0.0),
                                     _f(d, "sigma_yp", 0.0), dist, _f(d, "scale_parameter", 0.0)))
    continuous = [ContinuousPoint(_f(c, "energy"), _f(c, "horizontal_intensity"), _f(c, "vertical_intensity"),
                                  _f(c, "sigma_x", 0.0), _f(c, "sigma_xp", 0.0), _f(c, "sigma_y", 0.0),
                                  _f(c, "sigma_yp", 0.0)) for c in exc.findall("continuous")]
    exc_layers, det_layers = [], []
    if absb is not None:
        ep = absb.find("excitation_path")
        dp = absb.find("detector_path")
        exc_layers = [_layer(l) for l in ep.findall("layer")] if ep is not None else []
        det_layers = [_layer(l) for l in dp.findall("layer")] if dp is not None else []
    slit = geo.find("slit_size")
    return InputSpec(
        layers=layers, reference_layer=_f(comp, "reference_layer", cast=int),
        n_photons_interval=_f(g, "n_photons_interval", cast=int), n_photons_line=_f(g, "n_photons_line", cast=int),
        n_interactions_trajectory=_f(g, "n_interactions_trajectory", cast=int),
        d_sample_source=_f(geo, "d_sample_source"), n_sample_orientation=_xyz(geo, "n_sample_orientation"),
        p_detector_window=_xyz(geo, "p_detector_window"), n_detector_orientation=_xyz(geo, "n_detector_orientation"),
        area_detector=_f(geo, "area_detector"), collimator_height=_f(geo, "collimator_height", 0.0),
        collimator_diameter=_f(geo, "collimator_diameter", 0.0), d_source_slit=_f(geo, "d_source_slit"),
        slit_size_x=_f(slit, "slit_size_x"), slit_size_y=_f(slit, "slit_size_y"),
        discrete=discrete, continuous=continuous, exc_layers=exc_layers, det_layers=det_layers,
        detector_type=DETECTOR_TYPES.get(det.find("detector_type").text.strip(), 0),
        live_time=_f(det, "live_time"), pulse_width=_f(det, "pulse_width"),
        nchannels=_f(det, "nchannels", 2048, int), gain=_f(det, "gain"), zero=_f(det, "zero"),
        fano=_f(det, "fano"), noise=_f(det, "noise"),
        crystal_layers=[_layer(l) for l in det.find("crystal").findall("layer")])


def read_xmsi(path_or_text) -> InputSpec:
    text = Path(path_or_text).read_text() if not str(path_or_text).lstrip().startswith("<") else str(path_or_text)
    root = ET.fromstring(text)
    if root.tag == "xmimsim-results":
        root = root.find("xmimsim-input")
    return parse_input(root)


def _sub(parent, tag, text=None, **attrib):
    e = ET.SubElement(parent, tag, {k: str(v) for k, v in attrib.items()})
    if text is not None:
        e.text = text if isinstance(text, str) else ("%.10g" % text if isinstance(text, float) else str(text))
    return e


def _write_layer(parent, l: Layer):
    ln = _sub(parent, "layer")
    tot = float(sum(l.weight))
    for z, w in zip(l.Z, l.weight):
        el = _sub(ln, "element")
        _sub(el, "atomic_number", int(z))
        _sub(el, "weight_fraction", float(w) / tot * 100.0)
    _sub(ln, "density", float(l.density))
    _sub(ln, "thickness", float(l.thickness))


def input_element(s: InputSpec, tag: str = "xmimsim", outputfile: str = "") -> ET.Element:
    root = ET.Element(tag)
    g = _sub(root, "general", version="1.0")
    _sub(g, "outputfile", outputfile)
    _sub(g, "n_photons_interval", int(s.n_photons_interval))
    _sub(g, "n_photons_line", int(s.n_photons_line))
    _sub(g, "n_interactions_trajectory", int(s.n_interactions_trajectory))
    _sub(g, "comments", "")
    c = _sub(root, "composition")
    for l in s.layers:
        _write_layer(c, l)
    _sub(c, "reference_layer", int(s.reference_layer))
    geo = _sub(root, "geometry")
    _sub(geo, "d_sample_source", float(s.d_sample_source))
    for tag, v in (("n_sample_orientation", s.n_sample_orientation), ("p_detector_window", s.p_detector_window),
                   ("n_detector_orientation", s.n_detector_orientation)):
        e = _sub(geo, tag)
        for k, x in zip("xyz", v):
            _sub(e, k, float(x))
    _sub(geo, "area_detector", float(s.area_detector))
    _sub(geo, "collimator_height", float(s.collimator_height))
    _sub(geo, "collimator_diameter", float(s.collimator_diameter))
    _sub(geo, "d_source_slit", float(s.d_source_slit))
    sl = _sub(geo, "slit_size")
    _sub(sl, "slit_size_x", float(s.slit_size_x))
    _sub(sl, "slit_size_y", float(s.slit_size_y))
    exc = _sub(root, "excitation")
    inv_dist = {v: k for k, v in DIST_TYPES.items()}
    for d in s.discrete:
        e = _sub(exc, "discrete")
        for k in ("energy", "horizontal_intensity", "vertical_intensity", "sigma_x", "sigma_xp", "sigma_y",
                  "sigma_yp"):
            _sub(e, k, float(getattr(d, k)))
        if d.distribution_type != 0:
            _sub(e, "scale_parameter", float(d.scale_parameter), distribution_type=inv_dist[d.distribution_type])
    for cpt in s.continuous:
        e = _sub(exc, "continuous")
        for k in ("energy", "horizontal_intensity", "vertical_intensity", "sigma_x", "sigma_xp", "sigma_y",
                  "sigma_yp"):
            _sub(e, k, float(getattr(cpt, k)))
    ab = _sub(root, "absorbers")
    if s.exc_layers:
        ep = _sub(ab, "excitation_path")
        for l in s.exc_layers:
            _write_layer(ep, l)
    if s.det_layers:
        dp = _sub(ab, "detector_path")
        for l in s.det_layers:
            _write_layer(dp, l)
    det = _sub(root, "detector")
    _sub(det, "detector_type", {v: k for k, v in DETECTOR_TYPES.items()}[s.detector_type])
    _sub(det, "live_time", float(s.live_time))
    _sub(det, "pulse_width", float(s.pulse_width))
    _sub(det, "nchannels", int(s.nchannels))
    _sub(det, "gain", float(s.gain))
    _sub(det, "zero", float(s.zero))
    _sub(det, "fano", float(s.fano))
    _sub(det, "noise", float(s.noise))
    cr = _sub(det, "crystal")
    for l in s.crystal_layers:
        _write_layer(cr, l)
    return root


def write_xmsi(s: InputSpec, path) -> None:
    root = input_element(s)
    ET.indent(root)
    Path(path).write_text('<?xml version="1.0"?>\n' + ET.tostring(root, encoding="unicode") + "\n")


def _history_element(parent, tag, hist: np.ndarray | None, line_names, line_energy):
    h = _sub(parent, tag)
    if hist is None:
        return
    N = hist.shape[2]
    for Z in range(1, 101):
        block = hist[Z - 1, :383, :]
        tot = float(block.sum())
        if tot == 0.0:
            continue
        fl = _sub(h, "fluorescence_line_counts", atomic_number=Z, symbol=ELEMENT_SYMBOLS[Z - 1] if Z <= 94 else "",
                  total_counts="%g" % tot)
        for j in range(383):
            lt = float(block[j].sum())
            if lt == 0.0:
                continue
            ln = _sub(fl, "fluorescence_line", type=line_names[j + 1], energy="%g" % line_energy(Z, j + 1),
                      total_counts="%g" % lt)
            for k in range(N):
                if block[j, k] > 0.0:
                    _sub(ln, "counts", "%g" % block[j, k], interaction_number=k + 1)


def write_xmso(path, s: InputSpec, channels_conv: np.ndarray, channels_unconv: np.ndarray,
               brute: np.ndarray, var_red: np.ndarray | None, line_names, line_energy, inputfile: str = "",
               use_zero_interactions: int = 0) -> None:
    """Writes an .xmso file (src/xmi_xml.c:1638); line_names/line_energy map line index -> name / keV."""
    root = ET.Element("xmimsim-results", {"version": "1.0"})
    _sub(root, "inputfile", inputfile)
    N = channels_unconv.shape[0] - 1
    for tag, arr in (("spectrum_conv", channels_conv), ("spectrum_unconv", channels_unconv)):
        sp = _sub(root, tag)
        for ch in range(arr.shape[1]):
            c = _sub(sp, "channel")
            _sub(c, "channelnr", ch)
            _sub(c, "energy", "%g" % (s.zero + s.gain * ch))
            for k in range(0 if use_zero_interactions else 1, N + 1):
                _sub(c, "counts", "%g" % arr[k, ch], interaction_number=k)
    _history_element(root, "brute_force_history", brute, line_names, line_energy)
    _history_element(root, "variance_reduction_history", var_red, line_names, line_energy)
    root.append(input_element(s, "xmimsim-input"))
    ET.indent(root)
    Path(path).write_text('<?xml version="1.0"?>\n' + ET.tostring(root, encoding="unicode") + "\n")


def read_xmso(path) -> dict:
    """Reads an .xmso: spectra [N+1, nch] (rows absent in the file are zero),
    histories {(Z, line_name): {interaction: counts}} and the embedded input."""
    root = ET.parse(path).getroot()
    spec = parse_input(root.find("xmimsim-input"))
    N = spec.n_interactions_trajectory
    out = {"input": spec}
    for tag in ("spectrum_conv", "spectrum_unconv"):
        chans = root.find(tag).findall("channel")
        arr = np.zeros((N + 1, len(chans)))
        for c in chans:
            nr = int(c.find("channelnr").text)
            for cnt in c.findall("counts"):
                arr[int(cnt.get("interaction_number")), nr] = float(cnt.text)
        out[tag] = arr
    for tag in ("brute_force_history", "variance_reduction_history"):
        h = {}
        node = root.find(tag)
        if node is not None:
            for flc in node.findall("fluorescence_line_counts"):
                Z = int(flc.get("atomic_number"))
                for fl in flc.findall("fluorescence_line"):
                    h[(Z, fl.get("type"))] = {int(c.get("interaction_number")): float(c.text)
                                              for c in fl.findall("counts")}
        out[tag] = h
    return out
