"""Build the native library and the headless driver, in tree.

    python cuda-to-sycl-nbody_gb300/build.py [-v] [-j JOBS]

Outputs (git-ignored):
    nbody_gb300/libnbody_gb300.so   the C ABI of include/nbody_gb300.h
    nbody_gb300/nbody_gb300         the headless no_render driver
    build/                          object files

CUDA sources are compiled for sm_103a only; host sources are compiled with
-ffp-contract=off so host arithmetic is the same on x86-64 and aarch64.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
INCLUDE = PKG.parent / "include"
BUILD = PKG / "build"
OUT = PKG / "nbody_gb300"
LIB = OUT / "libnbody_gb300.so"
DRIVER = OUT / "nbody_gb300"

CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
NVCC = str(CUDA_HOME / "bin" / "nvcc") if (CUDA_HOME / "bin" / "nvcc").exists() else "nvcc"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-ftz=true", "-Xcompiler", "-fPIC",
                     "-Xcompiler", "-ffp-contract=off"]
CXX_FLAGS = ["-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-Wall"]

LIB_CU = ["force_shapes_a.cu", "force_shapes_b.cu", "force_shapes_c.cu", "force_kernel.cu", "reference_order_kernel.cu", "peak_probe.cu",
          "aux_kernels.cu", "diag_kernels.cu", "adjoint_kernel.cu", "initgen.cu", "noalloc.cu",
          "render_kernels.cu"]
LIB_CPP = ["nbody_capi.cpp", "nbody_aux.cpp", "nbody_render.cpp", "worklist.cpp",
           "initial_conditions.cpp"]
DRIVER_CPP = ["simulator.cpp", "nbody_main.cpp"]


def _headers() -> list[Path]:
    return sorted(CSRC.glob("*.hpp")) + sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h"))


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _run(cmd: list[str], verbose: bool) -> None:
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}")
    if verbose and r.stdout.strip():
        print(r.stdout, flush=True)


def _compile(src: Path, verbose: bool) -> Path:
    obj = BUILD / (src.name + ".o")
    if not _stale(obj, [src] + _headers()):
        return obj
    inc = ["-I", str(INCLUDE), "-I", str(CSRC)]
    if src.suffix == ".cu":
        cmd = [NVCC] + NVCC_FLAGS + inc + ["-c", str(src), "-o", str(obj)]
    else:
        cxx = os.environ.get("CXX", "g++")
        cmd = [cxx] + CXX_FLAGS + inc + ["-I", str(CUDA_HOME / "include"), "-c", str(src),
                                         "-o", str(obj)]
    _run(cmd, verbose)
    return obj


def build(verbose: bool = False, jobs: int | None = None) -> Path:
    """Compile and link; returns the path of the shared library."""
    if shutil.which(NVCC) is None and not Path(NVCC).exists():
        raise RuntimeError("nvcc not found; set CUDA_HOME")
    BUILD.mkdir(parents=True, exist_ok=True)
    srcs = [CSRC / f for f in LIB_CU + LIB_CPP + DRIVER_CPP]
    jobs = jobs or min(len(srcs), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = dict(zip(srcs, ex.map(lambda s: _compile(s, verbose), srcs)))
    lib_objs = [objs[CSRC / f] for f in LIB_CU + LIB_CPP]
    if _stale(LIB, lib_objs):
        _run([NVCC] + ARCH + ["-shared", "--cudart", "static", "-o", str(LIB)]
             + [str(o) for o in lib_objs], verbose)
    drv_objs = [objs[CSRC / f] for f in DRIVER_CPP]
    if _stale(DRIVER, drv_objs + [LIB]):
        cxx = os.environ.get("CXX", "g++")
        _run([cxx, "-o", str(DRIVER)] + [str(o) for o in drv_objs]
             + ["-L", str(OUT), "-lnbody_gb300", "-Wl,-rpath,$ORIGIN"], verbose)
    return LIB


def main() -> int:
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("-v", "--verbose", action="store_true")
    ap.add_argument("-j", "--jobs", type=int, default=None)
    a = ap.parse_args()
    lib = build(verbose=a.verbose, jobs=a.jobs)
    print(f"built {lib}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
