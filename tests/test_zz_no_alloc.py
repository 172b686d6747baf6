"""The allocation-free detector convolution, for callers that cannot allocate
device memory when they convolve a spectrum (a real-time acquisition or
fitting loop under a device-memory budget fixed up front, or an application
whose GPU memory belongs to another allocator).

It is called through the C-ABI twice in a row on different spectra and each
result must equal the allocating entry point's, within the tolerance of the
other convolution tests (1e-9 relative).  Collected last so that a failure
here never hides the rest of the suite; passes alone or after other tests."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _spectra(nch, seed):
    rng = np.random.default_rng(seed)
    base = rng.gamma(2.0, 50.0, size=nch)
    for c in rng.choice(nch, size=6, replace=False):
        base[max(0, c - 3):c + 3] += rng.uniform(1e3, 1e5)
    return base


@pytest.mark.parametrize("poisson", [0, 1])
def test_noalloc_matches_allocating_entry_point_twice(poisson):
    """With Poisson noise on, both entry points draw channel i from the same
    per-channel stream of the same seed, so the counts are equal too."""
    from xmimsim_gb300 import Simulation, abi, configs, gpu_options
    lib = abi.load()
    f = lib.xmi_detector_convolute_spectrum_noalloc
    spec = configs.config1(n_photons_line=10)
    sim = Simulation(spec, options=dict(use_escape_peaks=0, use_sum_peaks=0, use_poisson=poisson,
                                        use_default_seeds=1), gpu=gpu_options(seed=0x5EED0001))
    nch = spec.nchannels
    for call, seed in enumerate((1, 2)):
        x = np.ascontiguousarray(_spectra(nch, seed))
        out = np.full(nch, np.nan)
        rv = f(sim.inputF, x.ctypes.data_as(abi.c_double_p), out.ctypes.data_as(abi.c_double_p),
               C.byref(sim.options))
        assert rv == 1, abi.last_error()
        ref_p = abi.c_double_p()
        lib.xmi_detector_convolute_spectrum(sim.inputF, x.ctypes.data_as(abi.c_double_p), C.byref(ref_p),
                                            C.byref(sim.options), None, 1)
        assert ref_p, abi.last_error()
        ref = np.ctypeslib.as_array(ref_p, (nch,)).copy()
        lib.xmi_free(C.cast(ref_p, C.c_void_p))
        assert np.isfinite(out).all()
        np.testing.assert_allclose(out, ref, rtol=1e-9, atol=1e-12 * ref.max(), err_msg="call %d" % call)
    sim.close()


def test_noalloc_rejects_unsupported_sizes_and_options():
    from xmimsim_gb300 import Simulation, abi, configs
    lib = abi.load()
    f = lib.xmi_detector_convolute_spectrum_noalloc
    spec = configs.config1(n_photons_line=10)
    spec.nchannels = 20000
    sim = Simulation(spec, options=dict(use_escape_peaks=0, use_sum_peaks=0))
    x = np.ones(spec.nchannels)
    out = np.zeros(spec.nchannels)
    assert f(sim.inputF, x.ctypes.data_as(abi.c_double_p), out.ctypes.data_as(abi.c_double_p),
             C.byref(sim.options)) == 0
    assert "exceed" in abi.last_error()
    sim.close()
    spec = configs.config1(n_photons_line=10)
    sim = Simulation(spec, options=dict(use_escape_peaks=1, use_sum_peaks=0))
    x = np.ones(spec.nchannels)
    out = np.zeros(spec.nchannels)
    assert f(sim.inputF, x.ctypes.data_as(abi.c_double_p), out.ctypes.data_as(abi.c_double_p),
             C.byref(sim.options)) == 0
    assert "escape" in abi.last_error()
    sim.close()
