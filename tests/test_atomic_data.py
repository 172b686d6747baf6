"""The atomic data source of the host tabulator (xmi_atomic_data): the
default table is the stand-in model, every entry reaches the tables, and the
source can only be changed before the first tables are built.  CPU only (the
tables and the FP64 oracle run on the host)."""
import ctypes as C
import json
import os
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]

# first-order K-line histories of O, S, Ca in the CaSO4 input, with the data
# source scaled by HALVE (FluorYield halved) or left as it is
SCRIPT = r'''
import ctypes as C, json, sys
sys.path.insert(0, %(root)r)
sys.path.insert(0, %(tests)r)
from xmimsim_gb300 import abi, Simulation, configs
from oracle import oracle_api as O
from test_oracle import _oracle_grid
lib = abi.load()
keep = []
if %(halve)r:
    table = abi.XmiAtomicData.from_buffer_copy(lib.xmi_get_atomic_data().contents)
    base = lib.xrl_FluorYield
    base.restype, base.argtypes = C.c_double, [C.c_int, C.c_int]
    f = abi.ATOMIC_DATA_FUNC["FluorYield"](lambda Z, s: 0.5 * base(Z, s))
    keep.append(f)
    table.FluorYield = f
    table.name = b"halved yields"
    assert lib.xmi_set_atomic_data(C.byref(table)) == 1, abi.last_error()
    assert lib.xmi_get_atomic_data().contents.name == b"halved yields"
spec = configs.caso4(n_photons_line=3000)
sim = Simulation(spec, options=dict(use_variance_reduction=1, use_escape_peaks=0, use_default_seeds=1))
_oracle_grid(sim, 32, 32, 500)
sim.prepare()
res = O.msim(sim.bundle_ptr(), 1, spec.nchannels)
lines = {Z: float(res["var_red"][Z - 1, 0:29, 0].sum()) for Z in (8, 16, 20)}
# once tables exist the source is fixed
refused = lib.xmi_set_atomic_data(None) == 0 and "built" in abi.last_error()
print(json.dumps({"lines": lines, "refused": refused}))
'''


def _run(halve: bool) -> dict:
    code = SCRIPT % {"root": str(ROOT), "tests": str(ROOT / "tests"), "halve": halve}
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600,
                         env=dict(os.environ, OMP_NUM_THREADS="4"))
    assert out.returncode == 0, out.stderr[-2000:]
    return json.loads(out.stdout.strip().splitlines()[-1])


def test_default_table_is_the_stand_in_model():
    from xmimsim_gb300 import abi
    import xmimsim_gb300.tube as tube
    lib = abi.load()
    xrl = tube._xrl()
    t = lib.xmi_get_atomic_data().contents
    assert b"xrlite" in t.name
    for Z in (8, 26, 79):
        for E in (2.0, 17.44, 60.0):
            assert t.CS_Total_Kissel(Z, E) == xrl.xrl_CS_Total_Kissel(Z, E)
        assert t.LineEnergy(Z, 3) == xrl.xrl_LineEnergy(Z, 3)
        assert t.FluorYield(Z, 0) == xrl.xrl_FluorYield(Z, 0)
    for name, _ in abi.ATOMIC_DATA_ENTRIES:
        assert getattr(t, name), name


def test_installed_source_reaches_the_tables():
    """With every K-shell fluorescence yield halved, the first-order K-line
    histories of the same photons (same seed) halve exactly: the estimator's
    line factor is yield x radiative rate, and nothing else of a first-order
    K line depends on the yields.  After the tables are built the source
    cannot be changed any more."""
    a, b = _run(False), _run(True)
    for Z in ("16", "20"):  # O K lines lie below the 1 keV floor
        assert a["lines"][Z] > 0
        assert b["lines"][Z] == pytest.approx(0.5 * a["lines"][Z], rel=1e-9), Z
    assert a["refused"] and b["refused"]


def test_incomplete_table_is_refused():
    code = r'''
import ctypes as C, sys
sys.path.insert(0, %r)
from xmimsim_gb300 import abi
lib = abi.load()
t = abi.XmiAtomicData.from_buffer_copy(lib.xmi_get_atomic_data().contents)
t.CS_Rayl = abi.ATOMIC_DATA_FUNC["CS_Rayl"]()
assert lib.xmi_set_atomic_data(C.byref(t)) == 0 and "every entry" in abi.last_error()
assert b"xrlite" in lib.xmi_get_atomic_data().contents.name
print("ok")
''' % str(ROOT)
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0 and out.stdout.strip().endswith("ok"), out.stderr[-2000:]
