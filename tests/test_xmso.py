"""The output side of the library surface on the CPU: the raw outputs of the
reference's srm1155 example (examples/srm1155.xmso, as the fixture
tests/golden/srm1155_output.json holds them) go back into the raw layouts
xmi_main_msim returns, through xmi_output_raw2struct and
xmi_output_write_to_xml_file, and are read back: the unpacked histories list
exactly the elements, lines and interaction numbers the reference's own file
lists, with the same counts; the spectra and histories read from the written
file are the fixture's, number for number; the embedded input is the input."""
import ctypes as C
import json
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"


def _raw_from_fixture():
    from xmimsim_gb300 import xmlio
    import xmimsim_gb300.tube as tube
    g = json.loads((GOLDEN / "srm1155.json").read_text())
    out = json.loads((GOLDEN / "srm1155_output.json").read_text())
    spec = xmlio.read_xmsi(g["xmsi"])
    N = out["n_interactions"]
    nch = spec.nchannels
    xrl = tube._xrl()
    raw = {}
    for tag in ("brute_force_history", "variance_reduction_history"):
        h = np.zeros((100, 385, N))
        for Z, name, counts in out["histories"][tag]:
            line = xrl.xrl_line_from_name(name.encode())
            assert 1 <= line <= 383, name
            for k, c in counts:
                h[Z - 1, line - 1, k - 1] = c
        raw[tag] = h
    unconv = np.zeros((N + 1, nch))
    conv = np.zeros((N + 1, nch))
    unconv[1:] = out["spectrum_unconv"]
    conv[1:] = out["spectrum_conv"]
    return spec, out, raw, unconv, conv


def _unpacked(hist_ptr, n):
    res = {}
    for i in range(n):
        fc = hist_ptr[i]
        tot = 0.0
        for j in range(fc.n_lines):
            ln = fc.lines[j]
            res[(fc.atomic_number, ln.line_type.decode())] = {ln.interactions[k].interaction_number:
                                                               ln.interactions[k].counts
                                                               for k in range(ln.n_interactions)}
            assert ln.total_counts == pytest.approx(sum(res[(fc.atomic_number, ln.line_type.decode())].values()),
                                                    rel=1e-12)
            tot += ln.total_counts
        assert fc.total_counts == pytest.approx(tot, rel=1e-12)
    return res


def test_raw2struct_and_xmso_round_trip(tmp_path):
    from xmimsim_gb300 import abi, xmlio
    lib = abi.load()
    spec, out, raw, unconv, conv = _raw_from_fixture()
    cin = spec.to_c()
    brute = np.ascontiguousarray(raw["brute_force_history"])
    vr = np.ascontiguousarray(raw["variance_reduction_history"])
    unc = np.ascontiguousarray(unconv)
    rows = [np.ascontiguousarray(conv[i]) for i in range(conv.shape[0])]
    conv_p = (abi.c_double_p * len(rows))(*[r.ctypes.data_as(abi.c_double_p) for r in rows])
    o = lib.xmi_output_raw2struct(C.byref(cin.input), brute.ctypes.data_as(abi.c_double_p),
                                  vr.ctypes.data_as(abi.c_double_p), conv_p, unc.ctypes.data_as(abi.c_double_p),
                                  b"srm1155.xmsi", 0)
    assert o, abi.last_error()
    oc = o.contents
    N = out["n_interactions"]
    assert oc.ninteractions == N and oc.use_zero_interactions == 0
    # the unpacked histories are the reference file's, entry for entry
    for tag, hp, n in (("brute_force_history", oc.brute_force_history, oc.nbrute_force_history),
                       ("variance_reduction_history", oc.var_red_history, oc.nvar_red_history)):
        got = _unpacked(hp, n)
        want = {(Z, name): {k: c for k, c in counts} for Z, name, counts in out["histories"][tag]}
        assert got == want, tag
        zs = [hp[i].atomic_number for i in range(n)]
        assert zs == sorted(zs)
    for i in range(1, N + 1):
        assert np.array_equal(np.ctypeslib.as_array(oc.channels_unconv[i], (spec.nchannels,)), unconv[i])
    # the written file reads back as the same output
    path = tmp_path / "srm1155_copy.xmso"
    assert lib.xmi_output_write_to_xml_file(o, str(path).encode(), None) == 1, abi.last_error()
    back = xmlio.read_xmso(path)
    np.testing.assert_array_equal(back["spectrum_unconv"], unconv)
    np.testing.assert_array_equal(back["spectrum_conv"], conv)
    for tag in ("brute_force_history", "variance_reduction_history"):
        want = {(Z, name): {k: c for k, c in counts} for Z, name, counts in out["histories"][tag]}
        assert back[tag] == want, tag
    b = back["input"]
    assert b.n_interactions_trajectory == spec.n_interactions_trajectory and b.nchannels == spec.nchannels
    assert [l.Z for l in b.layers] == [l.Z for l in spec.layers]
    for lb, ls in zip(b.layers, spec.layers):
        np.testing.assert_allclose(np.array(lb.weight) / sum(lb.weight), np.array(ls.weight) / sum(ls.weight),
                                   rtol=1e-12)
        assert lb.thickness == ls.thickness and lb.density == ls.density
    assert b.gain == spec.gain and b.live_time == spec.live_time
    assert [d.energy for d in b.discrete] == [d.energy for d in spec.discrete]
    assert len(b.continuous) == len(spec.continuous)
    text = path.read_text()
    assert text.startswith('<?xml version="1.0"') and "<!DOCTYPE xmimsim-results" in text
    lib.xmi_output_free(o)


def test_raw2struct_without_variance_reduction():
    """Without a variance-reduction history (VR off) only the brute-force
    history is unpacked, as the reference does."""
    from xmimsim_gb300 import abi
    lib = abi.load()
    spec, out, raw, unconv, conv = _raw_from_fixture()
    cin = spec.to_c()
    brute = np.ascontiguousarray(raw["brute_force_history"])
    unc = np.ascontiguousarray(unconv)
    o = lib.xmi_output_raw2struct(C.byref(cin.input), brute.ctypes.data_as(abi.c_double_p), None, None,
                                  unc.ctypes.data_as(abi.c_double_p), None, 0)
    assert o and o.contents.nvar_red_history == 0 and not o.contents.var_red_history
    assert o.contents.nbrute_force_history == len({Z for Z, _, _ in out["histories"]["brute_force_history"]})
    lib.xmi_output_free(o)
