"""Generates the golden fixtures of tests/golden from the reference's own files.

Run once where the reference tree is available (it is not on the GPU
machines); the outputs are committed:

* xmi_lines.json      -- the line-name table of src/xmi_lines.c (history layout)
* quadratic.json      -- the (a, b, c) cases of tests/test-poly-solve-quadratic.F90
                         with the roots of GSL's gsl_poly_solve_quadratic (the
                         reference test's comparison target, tolerance 1e-7)
* srm1155.json        -- examples/srm1155.xmsi detector/input parameters and the
                         unconvolved and convolved spectra of examples/srm1155.xmso,
                         the input of tests/test-pile-up.c
* philox_kat.json     -- Philox4x32-10 known-answer vectors published with
                         Random123 (Salmon et al., SC'11)

usage: python tests/golden/make_golden.py <reference-root>
"""
from __future__ import annotations

import json
import math
import re
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))


def gsl_quadratic(a, b, c):
    """Restatement of gsl_poly_solve_quadratic (GSL 2.x, poly/solve_quadratic.c)."""
    if a == 0.0:
        if b == 0.0:
            return 0, None, None
        return 1, -c / b, None
    disc = b * b - 4 * a * c
    if disc > 0:
        if b == 0:
            r = math.sqrt(-c / a)
            return 2, -r, r
        sgnb = 1 if b > 0 else -1
        temp = -0.5 * (b + sgnb * math.sqrt(disc))
        r1, r2 = temp / a, c / temp
        return 2, min(r1, r2), max(r1, r2)
    if disc == 0:
        return 2, -0.5 * b / a, -0.5 * b / a
    return 0, None, None


def main(ref: Path) -> None:
    text = (ref / "src/xmi_lines.c").read_text()
    body = text[text.index("{") + 1: text.index("};")]
    names = re.findall(r'"([^"]*)"', body)
    assert len(names) == 386, len(names)
    (HERE / "xmi_lines.json").write_text(json.dumps({"source": "src/xmi_lines.c", "names": names}) + "\n")

    f90 = (ref / "tests/test-poly-solve-quadratic.F90").read_text()
    arrays = {}
    for var in "abc":
        m = re.search(r"REAL \(C_DOUBLE\), DIMENSION\(10\) :: %s = \[([^\]]*)\]" % var, f90)
        arrays[var] = [float(x.strip().replace("E", "e")) for x in m.group(1).split(",")]
    cases = []
    for a, b, c in zip(arrays["a"], arrays["b"], arrays["c"]):
        n, r1, r2 = gsl_quadratic(a, b, c)
        cases.append({"a": a, "b": b, "c": c, "n": n, "r1": r1, "r2": r2})
    (HERE / "quadratic.json").write_text(json.dumps({"source": "tests/test-poly-solve-quadratic.F90",
                                                     "tolerance": 1e-7, "cases": cases}, indent=1) + "\n")

    from xmimsim_gb300 import xmlio
    xmso = xmlio.read_xmso(ref / "examples/srm1155.xmso")
    spec = xmlio.read_xmsi(ref / "examples/srm1155.xmsi")
    N = spec.n_interactions_trajectory
    xmsi_text = (ref / "examples/srm1155.xmsi").read_text()
    (HERE / "srm1155.json").write_text(json.dumps({
        "source": "examples/srm1155.xmsi, examples/srm1155.xmso (tests/test-pile-up.c)",
        "xmsi": xmsi_text,
        "n_interactions": N,
        "unconv_last": xmso["spectrum_unconv"][N].tolist(),
        "conv_last": xmso["spectrum_conv"][N].tolist(),
        "pileup_channel": 1077, "pileup_min_ratio": 100.0}) + "\n")

    # the whole output of the srm1155 example: spectra of every order and both
    # histories, for the round trip through the library's output writer
    hist = {}
    for tag in ("brute_force_history", "variance_reduction_history"):
        hist[tag] = [[Z, name, sorted([int(k), c] for k, c in counts.items())]
                     for (Z, name), counts in sorted(xmso[tag].items())]
    (HERE / "srm1155_output.json").write_text(json.dumps({
        "source": "examples/srm1155.xmso",
        "n_interactions": N,
        "spectrum_conv": xmso["spectrum_conv"][1:].tolist(),
        "spectrum_unconv": xmso["spectrum_unconv"][1:].tolist(),
        "histories": hist}) + "\n")

    kat = [{"ctr": [0, 0, 0, 0], "key": [0, 0], "out": [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]},
           {"ctr": [0xffffffff] * 4, "key": [0xffffffff] * 2,
            "out": [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]},
           {"ctr": [0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344], "key": [0xa4093822, 0x299f31d0],
            "out": [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]}]
    (HERE / "philox_kat.json").write_text(json.dumps({"source": "Random123 kat_vectors, philox4x32 10 rounds",
                                                      "vectors": kat}, indent=1) + "\n")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of the xmimsim source tree>")
    main(Path(sys.argv[1]))
