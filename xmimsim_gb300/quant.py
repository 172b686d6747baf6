"""Quantification loop of ``xmimsim-pymca`` (bin/xmimsim-pymca.c:597-820)
on the batched engine.

A sample is quantified by iterating: simulate the measurement with the
current weight fractions of the quantified elements, compare each element's
simulated K-alpha (KL2 + KL3) or L-alpha (L3M4 + L3M5) intensity of the
variance-reduction histories, times the detector window and crystal
absorption (calculate_detector_absorption, bin/xmimsim-pymca.c:52-68), with
the measured net intensity, scale the weight by measured / simulated within
the reference's concentration-dependent jump limit, and rebuild the layer
from the matrix and the new weights (xmi_ilay_composition_pymca,
src/xmi_pymca.c:1647-1830).  The loop ends when the sums over elements of
((measured - simulated) / measured)^2 fall to 1e-3 for the K and the L
elements (XMI_PYMCA_CONV_THRESHOLD, at most XMI_PYMCA_MAX_ITERATIONS = 100
iterations, start concentration 1e-4; include/xmi_pymca.h:28-30).

Where the reference runs one sample's iterations one after the other,
``quantify`` runs many samples at once: each iteration simulates every sample
that has not converged in one ``xmi_main_msim_batch`` launch sequence.  Like
the reference, each sample's solid-angle grid is computed once, for its
starting composition, and reused in every iteration.

Not restated: reading a PyMca fit file (the measured intensities, matrix and
quantified elements are given directly), and the optional Rayleigh- and
ROI-normalisation modes of the reference loop.  One departure: the simulated
intensity sums the orders 1..N of the history; the reference's loop runs
k = 0..N through a 1-based index macro and so also reads the entry before the
first order (the previous line's last order).
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field
from typing import Sequence

import numpy as np

from . import abi
from .simulation import InputSpec, Layer, Simulation, XmiError

START_CONC = 0.0001
MAX_ITERATIONS = 100
CONV_THRESHOLD = 0.001

K_ALPHA = ("KL2", "KL3")
L_ALPHA = ("L3M4", "L3M5")


@dataclass
class QuantSample:
    """One measurement to quantify.

    spec: geometry, excitation and detector of the measurement; its layer
    ``ilay`` (0-based) is rebuilt from ``matrix`` and the quantified elements
    every iteration.  k_exp / l_exp: measured net K-alpha / L-alpha intensity
    of each element of ``z_quant`` (the one used is the first that is > 0, as
    in the reference).  reference / usematrix: a matrix element whose weight
    is kept fixed (PyMca's reference element).  weights: start
    concentrations (default START_CONC)."""
    spec: InputSpec
    ilay: int
    matrix: Layer
    z_quant: list[int]
    k_exp: list[float]
    l_exp: list[float]
    reference: int = 0
    usematrix: bool = False
    weights: list[float] | None = None


@dataclass
class QuantResult:
    weights: np.ndarray            # final weight fractions of z_quant
    layer: Layer                   # the quantified layer of the last iteration
    iterations: int
    converged: bool
    sum_k: float
    sum_l: float
    k_sim: np.ndarray = field(default_factory=lambda: np.zeros(0))
    l_sim: np.ndarray = field(default_factory=lambda: np.zeros(0))


def max_scale(weight: float) -> float:
    """The largest factor a weight may grow by in one iteration
    (bin/xmimsim-pymca.c:697-721)."""
    for lim, m in ((0.0001, 100.0), (0.01, 10.0), (0.1, 2.5), (0.25, 1.5), (0.375, 1.2), (0.50, 1.1),
                   (0.6, 1.05), (0.7, 1.025)):
        if weight <= lim:
            return m
    return 1.01


def layer_composition(matrix: Layer, z_quant: Sequence[int], weights: np.ndarray, reference: int = 0,
                      usematrix: bool = False, k_exp: Sequence[float] | None = None,
                      l_exp: Sequence[float] | None = None) -> Layer:
    """xmi_ilay_composition_pymca (src/xmi_pymca.c:1647-1830): the matrix
    elements scaled to what the quantified elements leave, the quantified
    elements at their weights, sorted by Z.  When the quantified weights and
    the reference element exceed 1, the weights up to and including the largest
    one (ties: the larger measured intensity) are scaled so that the total is 1
    and the matrix gets nothing.  ``weights`` is updated in place as in the
    reference."""
    m_w = np.asarray(matrix.weight, dtype=np.float64)
    m_w = m_w / m_w.sum()
    ref_w = 0.0
    if usematrix:
        for z, w in zip(matrix.Z, m_w):
            if z == reference:
                ref_w = float(w)
                break
    sum_quant = float(np.sum(weights))
    if sum_quant + ref_w > 1.0:
        maxval = float(np.max(weights))
        maxloc = int(np.argmax(weights))
        net = [(k if k > 0.0 else l) for k, l in zip(k_exp or [0.0] * len(weights), l_exp or [0.0] * len(weights))]
        best = net[maxloc]
        for i, w in enumerate(weights):
            if w == maxval and i != maxloc and net[i] > best:
                best, maxloc = net[i], i
        if maxval > 1.0:
            raise XmiError("layer_composition: a weight fraction above 1")
        sum_above = float(np.sum(weights[:maxloc + 1]))
        weights[:maxloc + 1] *= (1.0 - (sum_quant - sum_above) - ref_w) / sum_above
        sum_quant = 1.0 - ref_w
    Z, W = [], []
    for z, w in zip(matrix.Z, m_w):
        Z.append(int(z))
        W.append(ref_w if (usematrix and z == reference) else float(w) * (1.0 - sum_quant - ref_w) / (1.0 - ref_w))
    for z, w in zip(z_quant, weights):
        if w < 0.0:
            raise XmiError("layer_composition: negative weight fraction")
        Z.append(int(z))
        W.append(float(w))
    if min(W) < 0.0:
        raise XmiError("layer_composition: negative weight fraction")
    order = np.argsort(np.asarray(Z), kind="stable")
    return Layer([Z[i] for i in order], [W[i] for i in order], matrix.density, matrix.thickness)


def _xrl():
    lib = abi.load()
    lib.xrl_CS_Total_Kissel.restype = C.c_double
    lib.xrl_CS_Total_Kissel.argtypes = [C.c_int, C.c_double]
    lib.xrl_LineEnergy.restype = C.c_double
    lib.xrl_LineEnergy.argtypes = [C.c_int, C.c_int]
    lib.xrl_line_from_name.restype = C.c_int
    lib.xrl_line_from_name.argtypes = [C.c_char_p]
    return lib


def detector_absorption(spec: InputSpec, Z: int, line: str) -> float:
    """calculate_detector_absorption (bin/xmimsim-pymca.c:52-68): window and
    absorber transmission times crystal absorption at the line's energy."""
    lib = _xrl()
    E = lib.xrl_LineEnergy(Z, lib.xrl_line_from_name(line.encode()))
    rv = 1.0
    for lay in spec.det_layers:
        mu = sum(lib.xrl_CS_Total_Kissel(z, E) * w for z, w in zip(lay.Z, lay.weight))
        rv *= math.exp(-1.0 * lay.density * lay.thickness * mu)
    for lay in spec.crystal_layers:
        mu = sum(lib.xrl_CS_Total_Kissel(z, E) * w for z, w in zip(lay.Z, lay.weight))
        rv *= -1.0 * math.expm1(-1.0 * lay.density * lay.thickness * mu)
    return rv


def _simulated_alpha(out: dict, spec: InputSpec, Z: int, lines: Sequence[str]) -> float:
    lib = _xrl()
    v = 0.0
    for name in lines:
        idx = lib.xrl_line_from_name(name.encode())
        v += float(out["var_red"][Z - 1, idx - 1, :].sum()) * detector_absorption(spec, Z, name)
    return v


class _State:
    def __init__(self, s: QuantSample):
        self.s = s
        n = len(s.z_quant)
        self.weights = np.array(s.weights if s.weights is not None else [START_CONC] * n, dtype=np.float64)
        self.scale = np.ones(n)
        self.sum_k = self.sum_l = CONV_THRESHOLD * 10.0
        self.it = 0
        self.grid = None
        self.k_sim = np.zeros(n)
        self.l_sim = np.zeros(n)
        self.layer = layer_composition(s.matrix, s.z_quant, self.weights, s.reference, s.usematrix, s.k_exp, s.l_exp)

    def done(self) -> bool:
        return not (self.sum_k > CONV_THRESHOLD or self.sum_l > CONV_THRESHOLD)

    def spec_now(self) -> InputSpec:
        import copy
        spec = copy.deepcopy(self.s.spec)
        spec.layers = list(spec.layers)
        spec.layers[self.s.ilay] = self.layer
        return spec

    def update(self, out: dict) -> None:
        """One pass of the weight update of bin/xmimsim-pymca.c:652-770."""
        s = self.s
        self.sum_k = self.sum_l = 0.0
        for j, Z in enumerate(s.z_quant):
            self.k_sim[j] = _simulated_alpha(out, s.spec, Z, K_ALPHA)
            self.l_sim[j] = _simulated_alpha(out, s.spec, Z, L_ALPHA)
            if s.k_exp[j] > 0.0 and self.k_sim[j] > 0.0:
                self.scale[j] = s.k_exp[j] / self.k_sim[j]
            elif s.l_exp[j] > 0.0 and self.l_sim[j] > 0.0:
                self.scale[j] = s.l_exp[j] / self.l_sim[j]
        for j in range(len(s.z_quant)):
            ms = max_scale(self.weights[j])
            if s.k_exp[j] > 0.0 and self.k_sim[j] > 0.0:
                self.sum_k += (s.k_exp[j] - self.k_sim[j]) ** 2 / s.k_exp[j] / s.k_exp[j]
                self.weights[j] *= ms if self.scale[j] > ms else self.scale[j]
            elif s.l_exp[j] > 0.0 and self.l_sim[j] > 0.0:
                self.sum_l += (s.l_exp[j] - self.l_sim[j]) ** 2 / s.l_exp[j] / s.l_exp[j]
                self.weights[j] *= ms if self.scale[j] > ms else self.scale[j]
        self.layer = layer_composition(s.matrix, s.z_quant, self.weights, s.reference, s.usematrix, s.k_exp, s.l_exp)


def quantify(samples: Sequence[QuantSample], options: dict | None = None, gpu=None,
             max_iterations: int = MAX_ITERATIONS, strict: bool = False) -> list[QuantResult]:
    """Quantifies every sample; each iteration simulates all samples that have
    not converged in one batched call.  options: xmi_main_options fields
    (variance reduction must be on: the loop reads its histories); gpu:
    xmi_gpu_options for every simulation.

    A sample that has not converged after max_iterations stops there and is
    returned with converged = False while the others go on: the reference
    quantifies one sample per process and gives up on that sample alone
    (bin/xmimsim-pymca.c:602-605).  strict=True raises XmiError instead, once
    every sample has stopped."""
    opts = dict(options or {})
    if opts.get("use_variance_reduction", 1) != 1:
        raise XmiError("quantify: the loop reads the variance-reduction histories (use_variance_reduction = 1)")
    states = [_State(s) for s in samples]
    while True:
        active = [st for st in states if not st.done() and st.it < max_iterations]
        if not active:
            break
        for st in active:
            st.it += 1
        sims = []
        try:
            for st in active:
                sim = Simulation(st.spec_now(), options=opts, gpu=gpu)
                if st.grid is None:
                    st.grid = sim.solid_angle_grid()
                else:
                    sim.set_solid_angle(st.grid["r"], st.grid["theta"], st.grid["grid"])
                sims.append(sim)
            outs = Simulation.msim_batch(sims)
            for st, sim, out in zip(active, sims, outs):
                st.update(out)
                sim.free_raw(out)
        finally:
            for sim in sims:
                sim.close()
    if strict:
        failed = [i for i, st in enumerate(states) if not st.done()]
        if failed:
            raise XmiError(f"quantify: samples {failed} did not converge in {max_iterations} iterations")
    return [QuantResult(st.weights.copy(), st.layer, st.it, st.done(), st.sum_k, st.sum_l, st.k_sim.copy(),
                        st.l_sim.copy()) for st in states]
