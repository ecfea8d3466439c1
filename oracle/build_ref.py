"""Recipe for oracle/_ref: the reference's own host sources compiled in place
from the VisACD tree (never copied), with the stand-in headers of
oracle/ref_stubs for its absent third-party libraries, linked with
ref_shim.cpp / ref_bridge.cpp, the oracle and this project's remesh, hull and
cap-triangulation sources. Runs only where the reference tree exists (the
development container); the GPU machine uses fixtures generated from it.
Output: oracle/_ref/libvisacd_ref.so. TEST INFRASTRUCTURE ONLY."""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
REF = Path(os.environ.get("VISACD_REFERENCE_TREE", "/root/reference"))
OUT = HERE / "_ref"
LIB = OUT / "libvisacd_ref.so"
REF_SOURCES = ["clip.cpp", "core.cpp", "cost.cpp", "postprocess.cpp", "process.cpp",
               "support_surface.cpp"]
HOST = ROOT / "visacd_gb300" / "csrc" / "host"
PRODUCT_SOURCES = ["remesh.cpp", "hull.cpp", "core.cpp", "cap2d.cpp"]
FLAGS = ["-O2", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", "-w"]


def available() -> bool:
    return (REF / "lib" / "src" / "process.cpp").exists()


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"{' '.join(cmd)}\n{r.stderr[-4000:]}")


def build(force: bool = False) -> Path | None:
    if not available():
        return None
    OUT.mkdir(exist_ok=True)
    lib = REF / "lib"
    ref_inc = ["-I" + str(HERE / "ref_stubs"), "-I" + str(lib / "include"),
               "-I" + str(lib / "3rd" / "btConvexHull"), "-I" + str(lib / "3rd" / "quickhull")]
    jobs, objs = [], []
    for s in REF_SOURCES:
        o = OUT / ("ref_" + s.replace(".cpp", ".o"))
        objs.append(o)
        jobs.append(["g++", *FLAGS, *ref_inc, "-c", str(lib / "src" / s), "-o", str(o)])
    for s in ["btConvexHullComputer.cpp", "btAlignedAllocator.cpp"]:
        o = OUT / ("bt_" + s.replace(".cpp", ".o"))
        objs.append(o)
        jobs.append(["g++", *FLAGS, *ref_inc, "-c", str(lib / "3rd" / "btConvexHull" / s), "-o", str(o)])
    o = OUT / "qh_QuickHull.o"
    objs.append(o)
    jobs.append(["g++", *FLAGS, *ref_inc, "-c", str(lib / "3rd" / "quickhull" / "QuickHull.cpp"), "-o", str(o)])
    o = OUT / "ref_shim.o"
    objs.append(o)
    jobs.append(["g++", *FLAGS, *ref_inc, "-c", str(HERE / "ref_shim.cpp"), "-o", str(o)])
    for s in PRODUCT_SOURCES:
        o = OUT / ("prod_" + s.replace(".cpp", ".o"))
        objs.append(o)
        jobs.append(["g++", *FLAGS, "-I" + str(HOST), "-c", str(HOST / s), "-o", str(o)])
    o = OUT / "prod_ref_bridge.o"
    objs.append(o)
    jobs.append(["g++", *FLAGS, "-I" + str(HOST), "-c", str(HERE / "ref_bridge.cpp"), "-o", str(o)])
    o = OUT / "oracle.o"
    objs.append(o)
    jobs.append(["g++", *FLAGS, "-c", str(HERE / "visacd_oracle.cpp"), "-o", str(o)])
    deps = [HERE / "ref_shim.cpp", HERE / "ref_bridge.cpp", HERE / "visacd_oracle.cpp",
            *[HOST / s for s in PRODUCT_SOURCES], *sorted((HERE / "ref_stubs").rglob("*.h*"))]
    if not force and LIB.exists() and all(d.stat().st_mtime < LIB.stat().st_mtime for d in deps):
        return LIB
    with cf.ThreadPoolExecutor(max_workers=8) as ex:
        list(ex.map(_run, jobs))
    _run(["g++", "-shared", "-fopenmp", "-o", str(LIB), *map(str, objs)])
    return LIB


CUBIN = OUT / "ref_plane_intersections.cubin"


def build_cubin(force: bool = False) -> Path | None:
    """The reference's scoring kernel (lib/cuda/plane_intersections.cu), device
    code only, compiled unchanged for sm_103a so the benchmark can time it on the
    same GPU with the same planes and edges."""
    src = REF / "lib" / "cuda" / "plane_intersections.cu"
    if not src.exists():
        return None
    OUT.mkdir(exist_ok=True)
    if force or not CUBIN.exists() or src.stat().st_mtime > CUBIN.stat().st_mtime:
        _run(["/usr/local/cuda/bin/nvcc", "-cubin", "-O3", "-gencode", "arch=compute_103a,code=sm_103a",
              "-o", str(CUBIN), str(src)])
    return CUBIN


if __name__ == "__main__":
    print(build(force=True))
    print(build_cubin(force=True))
