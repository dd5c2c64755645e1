"""In-tree build of the native libraries.

- ``plens_gb300/lib/libplens_host.so``: host setup chain (C++17, g++).
- ``plens_gb300/lib/libplens_gpu.so``: CUDA kernels + the C ABI of include/plens_gpu.h, compiled
  for sm_103a only (``-gencode arch=compute_103a,code=sm_103a``).
- ``plens_gb300/lib/plens_gpu.out``: the command-line driver (``plens_gpu.out <mapping degree>
  <fe degree>`` reading ``./input.prm``), the counterpart of the reference's ``plens.out``.

Translation units are compiled in parallel; a library is rebuilt only when a source or header is
newer than it.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "plens_gb300"
CSRC = PKG / "csrc"
LIB = PKG / "lib"
BUILD = PKG / "_build"
INCLUDE = ROOT / "include"

GENCODE = "arch=compute_103a,code=sm_103a"
CXXFLAGS = ["-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-fopenmp", "-Wall", "-Wno-unused-function"]

HOST_SRCS = ["host/expr_compile.cpp", "host/prm.cpp", "host/setup.cpp", "host/output.cpp", "host/capi.cpp"]
GPU_SRCS = ["gpu/plens_gpu.cu", "gpu/mlp.cu", "gpu/noalloc.cu", "gpu/geometry.cu"]
# kernels_inst.cu is compiled once per (P, precision)
GPU_INST = [(P, prec) for P in (2, 3, 4, 5, 6) for prec in ("fp64", "mixed")]
DRIVER_SRCS = ["host/plens_driver.cpp", "host/main.cpp"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return cand


def _cuda_home() -> Path:
    return Path(_nvcc()).resolve().parent.parent


def _newer(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps if d.exists())


def _headers() -> list[Path]:
    return list(INCLUDE.glob("*.h")) + list(CSRC.rglob("*.h")) + list(CSRC.rglob("*.cuh"))


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"build command failed ({proc.returncode}): {' '.join(cmd)}\n{proc.stdout}")
    if proc.stdout.strip() and os.environ.get("PLENS_BUILD_VERBOSE"):
        sys.stderr.write(proc.stdout)


def _compile_objects(srcs: list[str], compiler, tag: str) -> list[Path]:
    BUILD.mkdir(parents=True, exist_ok=True)
    jobs = []
    objs = []
    hdrs = _headers()
    for s in srcs:
        src = CSRC / s
        obj = BUILD / (tag + "_" + s.replace("/", "_") + ".o")
        objs.append(obj)
        if _newer(obj, [src] + hdrs):
            jobs.append(compiler(src, obj))
    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(_run, jobs))
    return objs


def build_host() -> Path:
    LIB.mkdir(parents=True, exist_ok=True)
    out = LIB / "libplens_host.so"
    objs = _compile_objects(
        HOST_SRCS,
        lambda src, obj: ["g++", *CXXFLAGS, f"-I{INCLUDE}", "-c", str(src), "-o", str(obj)],
        "host",
    )
    if _newer(out, objs):
        _run(["g++", "-shared", "-fopenmp", "-o", str(out), *map(str, objs)])
    return out


def build_gpu() -> Path:
    LIB.mkdir(parents=True, exist_ok=True)
    out = LIB / "libplens_gpu.so"
    nvcc = _nvcc()
    flags = [
        "-gencode", GENCODE, "-lineinfo", "-O3", "-std=c++17", "--expt-relaxed-constexpr",
        "-Xcompiler", "-fPIC", f"-I{INCLUDE}", "-Xptxas", "-warn-spills",
    ]
    objs = _compile_objects(
        GPU_SRCS,
        lambda src, obj: [nvcc, *flags, "-c", str(src), "-o", str(obj)],
        "gpu",
    )
    # per-instantiation objects of kernels_inst.cu, compiled in parallel
    src = CSRC / "gpu" / "kernels_inst.cu"
    hdrs = _headers()
    jobs = []
    for P, prec in GPU_INST:
        obj = BUILD / f"gpu_kernels_{prec}_{P}.o"
        objs.append(obj)
        if _newer(obj, [src] + hdrs):
            real = "double" if prec == "fp64" else "float"
            # The plain FP64 form is compiled without multiply-add contraction: it then rounds
            # every product and sum as written, like the reference's x86-64 build (which has no
            # FMA), and matches the oracle to ~1e-15 even in stretched curved cells where the
            # residual cancels by four orders of magnitude. The mixed form keeps FMA.
            # The mixed form's FP32 divisions and square roots use the approximate instructions
            # (2 ulp); the FP64 arithmetic is unaffected by these flags.
            extra = ["--fmad=false"] if prec == "fp64" else ["-prec-div=false", "-prec-sqrt=false"]
            jobs.append([nvcc, *flags, *extra, f"-DPLENS_P={P}", f"-DPLENS_REAL={real}",
                         f"-DPLENS_TABLE=table_{prec}_{P}", "-c", str(src), "-o", str(obj)])
    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(_run, jobs))
    if _newer(out, objs):
        _run([nvcc, "-shared", "-gencode", GENCODE, "-o", str(out), *map(str, objs), "-lcudart"])
    return out


def build_driver() -> Path:
    """Command-line driver linking both libraries (rpath to the in-tree lib directory)."""
    out = LIB / "plens_gpu.out"
    objs = _compile_objects(
        DRIVER_SRCS,
        lambda src, obj: ["g++", *CXXFLAGS, f"-I{INCLUDE}", "-c", str(src), "-o", str(obj)],
        "drv",
    )
    libs = [LIB / "libplens_host.so", LIB / "libplens_gpu.so"]
    if _newer(out, objs + libs):
        _run(["g++", "-fopenmp", "-o", str(out), *map(str, objs), f"-L{LIB}", "-lplens_host", "-lplens_gpu",
              f"-Wl,-rpath,{LIB}"])
    return out


def build_all(gpu: bool = True, driver: bool = True) -> dict[str, Path]:
    res = {"host": build_host()}
    if gpu:
        res["gpu"] = build_gpu()
        if driver:
            res["driver"] = build_driver()
    return res


if __name__ == "__main__":
    for k, v in build_all().items():
        print(k, v)
