"""Workload definitions: the benchmark configurations as seeded synthetic inputs.

* ``config1``: the small plain case (air + silicate sample, 17.44 keV mono, 45/45 deg,
  10 cm, 4 interactions, 1e5 photons) -- the reference default input
  (src/xmi_data_structs.c:551-640) with the changes named in the workload.
* ``config2``: the production-size plain case (5 random layers, Rh tube at
  40 kV through 125 um Be in 400 intervals plus the Rh K/L lines, 1e8 photons,
  6 interactions).
* ``caso4``: the reference's CaSO4 first-interaction test input
  (tests/libxmimsim-test.c:182-244).
"""
from __future__ import annotations

import math

import numpy as np

from .simulation import ContinuousPoint, DiscreteLine, InputSpec, Layer
from . import tube

AIR = Layer([7, 8, 18], [0.755, 0.232, 0.013], 1.2e-3, 5.0)


def config1(n_photons_line: int = 100000) -> InputSpec:
    sample = Layer([14, 8, 26, 29, 30], [0.40, 0.50, 0.05, 0.03, 0.02], 2.5, 0.1)
    return InputSpec(
        layers=[AIR, sample], reference_layer=2,
        n_photons_line=n_photons_line, n_interactions_trajectory=4,
        d_sample_source=100.0,
        n_sample_orientation=(0.0, -math.sqrt(2.0) / 2.0, math.sqrt(2.0) / 2.0),
        p_detector_window=(0.0, 10.0, 100.0), n_detector_orientation=(0.0, -1.0, 0.0),
        area_detector=0.3,
        discrete=[DiscreteLine(17.44, 1e9, 0.0)],
    )


C1_OPTIONS = dict(use_variance_reduction=1, use_escape_peaks=1, use_sum_peaks=0, use_M_lines=1,
                  use_cascade_auger=1, use_cascade_radiative=1, use_default_seeds=1)


def random_layers(seed: int, n_layers: int = 5, zmin: int = 6, zmax: int = 82, nel=(3, 12),
                  thick=(0.5e-4, 0.2), rho=(1.0, 8.0)) -> list[Layer]:
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n_layers):
        n = int(rng.integers(nel[0], nel[1] + 1))
        Z = sorted(rng.choice(np.arange(zmin, zmax + 1), size=n, replace=False).tolist())
        w = rng.dirichlet(np.ones(n)).tolist()
        t = float(np.exp(rng.uniform(np.log(thick[0]), np.log(thick[1]))))
        d = float(rng.uniform(*rho))
        out.append(Layer([int(z) for z in Z], w, d, t))
    return out


def config2(total_photons: int = 100_000_000, seed: int = 2) -> InputSpec:
    layers = random_layers(seed)
    cont, lines = tube.rh_tube_40kv(n_intervals=400)
    n_lines = len(lines)
    # n_photons_interval*400 + n_photons_line*n_lines ~ total, equal per-item counts
    per_item = total_photons // (400 + n_lines)
    return InputSpec(
        layers=layers, reference_layer=1,
        n_photons_interval=per_item, n_photons_line=per_item, n_interactions_trajectory=6,
        d_sample_source=100.0,
        n_sample_orientation=(0.0, -math.sqrt(2.0) / 2.0, math.sqrt(2.0) / 2.0),
        p_detector_window=(0.0, 10.0, 100.0), n_detector_orientation=(0.0, -1.0, 0.0),
        area_detector=0.3,
        discrete=lines, continuous=cont,
    )


C2_OPTIONS = dict(use_variance_reduction=1, use_escape_peaks=1, use_sum_peaks=1, use_M_lines=1,
                  use_cascade_auger=1, use_cascade_radiative=1, use_default_seeds=1)


def caso4(n_photons_line: int = 1000000) -> InputSpec:
    # Ca S O4 by mass: Ca 40.078, S 32.06, O 4*15.999
    a = {20: 40.078, 16: 32.06, 8: 4 * 15.999}
    tot = sum(a.values())
    layer = Layer([8, 16, 20], [a[8] / tot, a[16] / tot, a[20] / tot], 1.0, 1.0)
    return InputSpec(layers=[layer], reference_layer=1, n_photons_line=n_photons_line,
                     n_interactions_trajectory=1, p_detector_window=(0.0, 10.0, 100.0),
                     discrete=[DiscreteLine(10.0, 1e12, 1e9)])
