"""Generates tests/golden/cl_solid_angle.json: solid angles computed by the
reference's own OpenCL solid-angle kernel (src/xmi_kernels.cl:219-453), run
on the host through oracle/_ref/libref_cl.so (built by oracle/ref_cl/Makefile
from the reference tree), at seeded random points of the 1024 x 1024 grid of
three geometries: no collimator and two conical collimators (the reference's
xmi_init_input accepts only conical ones, src/xmi_main.F90:1780-1796).

Stored per geometry: the geometry, the grid points (r index, theta index and
their FP32 axis values), the kernel's result, and the solid angle of the
point's sampling cone (restated below from the kernel's set-up lines, FP64)
so that a test can turn values back into hit counts out of 5000.  Also the
Threefry4x32-20 blocks of the reference's Random123 header for a few inputs.

usage (where the reference tree exists): make -C oracle/ref_cl REF=<tree> && python tests/golden/make_cl_solid_angle.py
"""
from __future__ import annotations

import json
import math
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))

N_POINTS = 600
HITS = 5000


def geometries():
    from xmimsim_gb300 import configs
    plain = configs.config1(n_photons_line=10)
    con = configs.config1(n_photons_line=10)
    con.collimator_height = 1.0
    con.collimator_diameter = 0.2
    wide = configs.config1(n_photons_line=10)
    wide.collimator_height = 0.5
    wide.collimator_diameter = 0.4
    return {"no_collimator": plain, "conical_collimator": con, "conical_collimator_wide": wide}


def cone_solid_angle(r1, theta1, present, detr, collr, collh):
    """FP64 restatement of the kernel's cone set-up (src/xmi_kernels.cl:284-335)."""
    if not present:
        r, theta, fcbr = r1, theta1, detr
    elif abs(collr - detr) < 1e-6:
        if r1 * math.cos(theta1) <= detr:
            r, theta, fcbr = r1, theta1, detr
        else:
            r = math.sqrt(r1 * r1 - 2.0 * r1 * math.sin(theta1) * collh + collh * collh)
            theta, fcbr = math.acos(r1 * math.cos(theta1) / r), collr
    else:
        if r1 * math.cos(theta1) <= detr and r1 * math.sin(theta1) <= collh * (r1 * math.cos(theta1) - detr) / (
                collr - detr):
            r, theta, fcbr = r1, theta1, detr
        elif r1 * math.sin(theta1) <= collh:
            return 0.0
        else:
            r = math.sqrt(r1 * r1 - 2.0 * r1 * math.sin(theta1) * collh + collh * collh)
            theta, fcbr = math.acos(r1 * math.cos(theta1) / r), collr
    beta = math.atan(fcbr / r)
    alpha1 = math.atan(fcbr * math.sin(theta) / (r - fcbr * math.cos(theta)))
    if alpha1 <= 0.0:
        alpha1 += math.pi
    return 2 * math.pi * (1.0 - math.cos(max(beta, alpha1)))


def main() -> None:
    from oracle import oracle_api
    from xmimsim_gb300 import Simulation
    out = {"hits_per_single": HITS, "source": "src/xmi_kernels.cl (reference OpenCL kernel run on the host)",
           "geometries": {}}
    rng = np.random.default_rng(20240601)
    for name, spec in geometries().items():
        sim = Simulation(spec, options=dict(use_variance_reduction=1, use_escape_peaks=0, use_default_seeds=1))
        r, t = sim.grid_axes(1024, 1024)
        detr = math.sqrt(spec.area_detector / math.pi)
        present = 1 if spec.collimator_height > 0 and spec.collimator_diameter > 0 else 0
        collr = spec.collimator_diameter / 2.0
        collh = spec.collimator_height
        ir = rng.integers(0, 1024, size=N_POINTS).astype(np.int32)
        it = rng.integers(0, 1024, size=N_POINTS).astype(np.int32)
        vals = oracle_api.ref_cl_solid_angle_points(r, t, ir, it, present, detr, collr, collh, HITS)
        r32, t32 = np.float32(r), np.float32(t)
        cone = [cone_solid_angle(float(r32[i]), float(t32[j]), present, float(np.float32(detr)),
                                 float(np.float32(collr)), float(np.float32(collh))) for i, j in zip(ir, it)]
        out["geometries"][name] = {
            "detector_radius": detr, "collimator_present": present, "collimator_radius": collr,
            "collimator_height": collh, "ir": ir.tolist(), "it": it.tolist(),
            "r": [float(x) for x in r32[ir]], "theta": [float(x) for x in t32[it]],
            "value": [float(x) for x in vals], "cone_solid_angle": cone}
        sim.close()
    kat = []
    for ctr, key in (([0, 0, 0, 0], [0, 0, 0, 0]), ([0xffffffff] * 4, [0xffffffff] * 4),
                     ([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344],
                      [0xa4093822, 0x299f31d0, 0x082efa98, 0xec4e6c89]),
                     ([1, 0xf00dcafe, 0xdeadbeef, 0xbeeff00d], [17, 0xdecafbad, 0xfacebead, 900])):
        kat.append({"ctr": ctr, "key": key, "out": oracle_api.ref_cl_threefry_block(ctr, key)})
    out["threefry4x32_20"] = kat
    (HERE / "cl_solid_angle.json").write_text(json.dumps(out, indent=0))
    print("wrote", HERE / "cl_solid_angle.json")


if __name__ == "__main__":
    main()
