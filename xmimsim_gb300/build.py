"""Build recipe of the engine library and of the CPU oracle.

Compiles, in parallel, the host C sources with gcc and the CUDA sources with
nvcc for sm_103a, links ``xmimsim_gb300/_lib/libxmimsim_gb300.so`` in-tree,
and builds the oracle (test infrastructure) into ``oracle/_build``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
LIBDIR = PKG / "_lib"
OBJDIR = ROOT / "_build" / "obj"
ORACLE = ROOT / "oracle"
ORACLE_BUILD = ORACLE / "_build"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CFLAGS = ["-std=gnu11", "-O2", "-fPIC", "-fopenmp", "-ffp-contract=off", "-Wall",
          "-Wno-unused-parameter", "-Wno-unused-function"]
NVFLAGS = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
                  "-Xcompiler", "-fopenmp"]

HOST_SOURCES = ["xrlite.c", "atomic_data.c", "host.c", "ebel.c", "xmso.c"]
CUDA_SOURCES = ["engine.cu", "detector.cu", "mlp.cu"]
ORACLE_SOURCES = ["oracle_transport.c", "oracle_detector.c"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the engine is CUDA-only and cannot be built")


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("build step failed: %s\n%s%s" % (" ".join(cmd), res.stdout, res.stderr))


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _deps() -> list[Path]:
    return sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.inc")) + \
        sorted((ROOT / "include").glob("*.h"))


def build_engine(verbose: bool = False, checked: bool = False) -> Path:
    """Compiles the engine and returns the path of the shared library.

    checked=True builds the diagnostic variant libxmimsim_gb300_checked.so in
    which every table load and tally store of the transport kernel is
    bounds-checked (violations are recorded, not executed)."""
    nvcc = _nvcc()
    objdir = OBJDIR / "checked" if checked else OBJDIR
    objdir.mkdir(parents=True, exist_ok=True)
    LIBDIR.mkdir(parents=True, exist_ok=True)
    nvflags = NVFLAGS + (["-DXMI_CHECKED"] if checked else [])
    deps = _deps()
    jobs = []
    objs = []
    for src in HOST_SOURCES:
        obj = objdir / (src + ".o")
        objs.append(obj)
        if _stale(obj, deps + [CSRC / src]):
            jobs.append(["gcc", *CFLAGS, "-c", str(CSRC / src), "-o", str(obj)])
    for src in CUDA_SOURCES:
        obj = objdir / (src + ".o")
        objs.append(obj)
        if _stale(obj, deps + [CSRC / src]):
            jobs.append([nvcc, *nvflags, "-c", str(CSRC / src), "-o", str(obj)])
    with cf.ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        list(ex.map(_run, jobs))
    lib = LIBDIR / ("libxmimsim_gb300_checked.so" if checked else "libxmimsim_gb300.so")
    if _stale(lib, objs):
        _run([nvcc, *ARCH, "-shared", "-Xcompiler", "-fopenmp", "-o", str(lib), *map(str, objs),
              "-lgomp", "-lm"])
    if verbose:
        print("built", lib)
    return lib


def build_oracle(verbose: bool = False) -> Path:
    """Compiles the FP64 CPU oracle (test infrastructure) into oracle/_build."""
    ORACLE_BUILD.mkdir(parents=True, exist_ok=True)
    lib = ORACLE_BUILD / "liboracle_xmimsim.so"
    srcs = [ORACLE / s for s in ORACLE_SOURCES]
    deps = srcs + sorted(ORACLE.glob("*.h")) + sorted((ROOT / "include").glob("*.h"))
    if _stale(lib, deps):
        _run(["gcc", *CFLAGS, "-O3", "-shared", "-o", str(lib), *map(str, srcs), "-lm"])
    if verbose:
        print("built", lib)
    return lib


# where the reference source tree is mounted in the build container; absent on
# GPU machines, where the reference's own OpenCL kernel is not built
REFERENCE_TREE = Path("/root/reference")


def build_reference_kernel(verbose: bool = False) -> Path | None:
    """Compiles the reference's OpenCL solid-angle kernel as host code into
    oracle/_ref (test infrastructure: it generates the golden fixture of the
    grid) when the reference tree is present; returns None otherwise."""
    if not (REFERENCE_TREE / "src" / "xmi_kernels.cl").exists() or shutil.which("make") is None:
        return None
    _run(["make", "-s", "-C", str(ORACLE / "ref_cl"), "REF=%s" % REFERENCE_TREE])
    lib = ORACLE / "_ref" / "libref_cl.so"
    if verbose:
        print("built", lib)
    return lib


def build_all(verbose: bool = False) -> None:
    with cf.ThreadPoolExecutor(max_workers=3) as ex:
        f1 = ex.submit(build_engine, verbose)
        f2 = ex.submit(build_oracle, verbose)
        f3 = ex.submit(build_reference_kernel, verbose)
        f1.result()
        f2.result()
        f3.result()


if __name__ == "__main__":
    build_all(verbose=True)
