"""Build recipe for the native parts: the sm_103a kernel library (C ABI) and the
pybind11 host module. Plain nvcc / g++ invocations, compiled in parallel, output
in-tree next to the sources (git-ignored). No cmake.

    python -m visacd_gb300.build          # build everything that is stale
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys
import sysconfig
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
INCLUDE = ROOT / "include"
GPU_SRC = PKG / "csrc" / "gpu"
HOST_SRC = PKG / "csrc" / "host"
BUILD = PKG / "_build"
GPU_LIB = PKG / "libvisacd_gpu.so"

NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", f"-I{INCLUDE}"]


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps if d.exists())


def build_gpu(force: bool = False) -> Path:
    """Compile csrc/gpu/*.cu for sm_103a into libvisacd_gpu.so."""
    BUILD.mkdir(exist_ok=True)
    sources = sorted(GPU_SRC.glob("*.cu"))
    headers = sorted(GPU_SRC.glob("*.cuh")) + [INCLUDE / "visacd_gpu.h"]
    objs = []
    jobs = []
    for s in sources:
        o = BUILD / (s.stem + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([NVCC, *NVCC_FLAGS, "-c", str(s), "-o", str(o)])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            list(ex.map(_run, jobs))
    if force or jobs or _stale(GPU_LIB, objs):
        _run([NVCC, *ARCH, "-shared", "-o", str(GPU_LIB), *map(str, objs)])
    return GPU_LIB


HOST_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", "-fvisibility=hidden"]


def _pybind_include() -> str:
    """pybind11 headers: the copy shipped with torch (present on every box) or
    the pybind11 package."""
    import importlib.util

    spec = importlib.util.find_spec("torch")
    if spec and spec.submodule_search_locations:
        inc = Path(list(spec.submodule_search_locations)[0]) / "include"
        if (inc / "pybind11" / "pybind11.h").exists():
            return str(inc)
    import pybind11  # noqa: WPS433

    return pybind11.get_include()


def host_module_path() -> Path:
    return PKG / ("visacd" + sysconfig.get_config_var("EXT_SUFFIX"))


def build_host(force: bool = False) -> Path:
    """Compile csrc/host/*.cpp into the pybind11 module `visacd` (linked to the
    kernel library through the C ABI)."""
    build_gpu(force)
    BUILD.mkdir(exist_ok=True)
    inc = ["-I" + str(INCLUDE), "-I" + sysconfig.get_paths()["include"], "-I" + _pybind_include()]
    sources = sorted(HOST_SRC.glob("*.cpp"))
    headers = sorted(HOST_SRC.glob("*.hpp")) + [INCLUDE / "visacd_gpu.h"]
    objs, jobs = [], []
    for s in sources:
        o = BUILD / ("host_" + s.stem + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append(["g++", *HOST_FLAGS, *inc, "-c", str(s), "-o", str(o)])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            list(ex.map(_run, jobs))
    out = host_module_path()
    if force or jobs or _stale(out, objs + [GPU_LIB]):
        _run(["g++", "-shared", "-fopenmp", "-o", str(out), *map(str, objs), f"-L{PKG}",
              "-lvisacd_gpu", "-Wl,-rpath,$ORIGIN"])
    return out


def build_all(force: bool = False) -> None:
    build_gpu(force)
    build_host(force)


if __name__ == "__main__":
    build_gpu(force="--force" in sys.argv)
    print(GPU_LIB)
