"""Workload definitions: the benchmark configurations as seeded synthetic inputs.

* ``config1``: the small plain case (air + silicate sample, 17.44 keV mono, 45/45 deg,
  10 cm, 4 interactions, 1e5 photons) -- the reference default input
  (src/xmi_data_structs.c:551-640) with the changes named in the workload.
* ``config2``: the production-size plain case (5 random layers, Rh tube at
  40 kV through 125 um Be in 400 intervals plus the Rh K/L lines, 1e8 photons,
  6 interactions).
* ``config3``: the precision form of config 1 (10 nm and 50 nm layers over a
  2 mm substrate).
* ``config4``: the learned solid-angle surrogate's workload (config 1 with a
  conical collimator, 1e8 photons).
* ``config5``: the 512-configuration batched quantification sweep.
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


def config3(n_photons_line: int = 100000) -> InputSpec:
    """The precision form of config 1: thin layers over a 2 mm substrate --
    10 nm of Cr (7.19 g/cm3) and 50 nm of Au (19.3 g/cm3) on the config-1
    sample 0.2 cm thick, behind the same 5 cm of air; the FP32 transport with
    FP64 plane heights must resolve the 10 nm layer 100 cm from the source."""
    spec = config1(n_photons_line=n_photons_line)
    sample = Layer([14, 8, 26, 29, 30], [0.40, 0.50, 0.05, 0.03, 0.02], 2.5, 0.2)
    spec.layers = [AIR, Layer([24], [1.0], 7.19, 1e-6), Layer([79], [1.0], 19.3, 5e-6), sample]
    spec.reference_layer = 2
    return spec


def config4(n_photons_line: int = 100_000_000) -> InputSpec:
    """The learned solid-angle surrogate's workload: the config-1 geometry
    with a conical collimator of height 1 cm and opening radius 0.1 cm
    (collimator_diameter 0.2) in front of the 0.3 cm2 detector (radius
    0.309 cm > 0.1 cm, so the conical case of src/xmi_main.F90:1780-1796),
    45/45 degrees, 10 cm from the sample, 1e8 photons."""
    spec = config1(n_photons_line=n_photons_line)
    spec.collimator_height = 1.0
    spec.collimator_diameter = 0.2
    return spec


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


def config5(n_configs: int = 512, seed: int = 5, budget_scale: float = 1.0) -> list[InputSpec]:
    """The batched quantification sweep: n_configs independent samples in the
    45/45 geometry of config 1 (detector 10 cm away, no collimator), 1-8
    layers of 2-20 elements whose weight fractions vary by +-20% around the
    config-1 sample (renormalised; extra elements drawn from Z 6-82 share
    the rest), mixed excitation (1-5 discrete lines or 50-400 continuous
    intervals of the Rh-tube spectrum), photon budgets log-uniform in
    [1e6, 1e8] (times budget_scale), 4 interactions."""
    rng = np.random.default_rng(seed)
    base_Z = [14, 8, 26, 29, 30]
    base_w = np.array([0.40, 0.50, 0.05, 0.03, 0.02])
    out = []
    for _ in range(n_configs):
        n_layers = int(rng.integers(1, 9))
        layers = []
        for _ in range(n_layers):
            n_el = int(rng.integers(2, 21))
            k = min(n_el, len(base_Z))
            Z = list(base_Z[:k])
            w = list(base_w[:k] * rng.uniform(0.8, 1.2, size=k))
            extra = [z for z in rng.permutation(np.arange(6, 83)).tolist() if z not in Z][:n_el - k]
            Z += extra
            w += list(rng.uniform(0.001, 0.02, size=len(extra)))
            w = np.array(w) / np.sum(w)
            order = np.argsort(Z)
            layers.append(Layer([int(Z[i]) for i in order], [float(w[i]) for i in order],
                                float(rng.uniform(1.0, 5.0)), float(np.exp(rng.uniform(np.log(1e-4), np.log(0.1))))))
        budget = int(np.exp(rng.uniform(np.log(1e6), np.log(1e8))) * budget_scale)
        if rng.uniform() < 0.5:
            n_lines = int(rng.integers(1, 6))
            energies = rng.uniform(8.0, 30.0, size=n_lines)
            disc = [DiscreteLine(float(e), 1e9, 1e7) for e in energies]
            spec = InputSpec(layers=layers, reference_layer=1, n_photons_line=max(1, budget // n_lines),
                             n_interactions_trajectory=4, discrete=disc, continuous=[],
                             p_detector_window=(0.0, 10.0, 100.0))
        else:
            n_int = int(rng.integers(50, 401))
            cont, lines = tube.rh_tube_40kv(n_intervals=n_int)
            spec = InputSpec(layers=layers, reference_layer=1,
                             n_photons_interval=max(1, budget // (n_int + len(lines))),
                             n_photons_line=max(1, budget // (n_int + len(lines))),
                             n_interactions_trajectory=4, discrete=lines, continuous=cont,
                             p_detector_window=(0.0, 10.0, 100.0))
        spec.n_sample_orientation = (0.0, -math.sqrt(2.0) / 2.0, math.sqrt(2.0) / 2.0)
        spec.n_detector_orientation = (0.0, -1.0, 0.0)
        out.append(spec)
    return out


C5_OPTIONS = dict(use_variance_reduction=1, use_escape_peaks=0, use_sum_peaks=0, use_M_lines=1,
                  use_cascade_auger=1, use_cascade_radiative=1, use_default_seeds=1)
