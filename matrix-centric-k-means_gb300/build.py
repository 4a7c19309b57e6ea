"""Builds libkm_sm103.so (CUDA kernels + C ABI, sm_103a), libkmeans_host.so
(the Kmeans class) and the gpukmeans CLI.

Every translation unit is compiled in parallel: .cu files by nvcc for
sm_103a only, .cpp files by g++.  Objects go to _build/, the library to lib/
(both git-ignored).  Run as a script or call build().
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
HOST = PKG / "host"
OBJ = PKG / "_build"
LIB = PKG / "lib"
LIBNAME = "libkm_sm103.so"

NVCC_FLAGS = [
    "-gencode", "arch=compute_103a,code=sm_103a",
    "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
    "-Xptxas", "-warn-spills",
]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-pthread", "-Wall"]


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and Path(c).exists():
            return c
    raise RuntimeError("nvcc not found")


def _cuda_home() -> Path:
    return Path(_nvcc()).resolve().parent.parent


def _run(cmd: list[str]) -> str:
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + p.stdout + p.stderr)
    return p.stdout + p.stderr


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, jobs: int | None = None) -> Path:
    """Compiles the library (incrementally) and returns its path."""
    OBJ.mkdir(exist_ok=True)
    LIB.mkdir(exist_ok=True)
    nvcc = _nvcc()
    inc = PKG.parent / "include"
    headers = sorted(CSRC.glob("*.cuh")) + sorted(inc.glob("*.h"))
    cus = sorted(CSRC.glob("*.cu"))
    cpps = sorted(CSRC.glob("*.cpp"))
    jobs_list = []
    for src in cus:
        out = OBJ / (src.stem + ".o")
        if _stale(out, [src] + headers):
            jobs_list.append([nvcc, *NVCC_FLAGS, "-I", str(inc), "-c", str(src), "-o", str(out)])
    for src in cpps:
        out = OBJ / (src.stem + ".cpp.o")
        if _stale(out, [src] + headers):
            jobs_list.append(["g++", *CXX_FLAGS, "-I", str(inc), "-c", str(src), "-o", str(out)])
    logs = []
    if jobs_list:
        with cf.ThreadPoolExecutor(max_workers=jobs or min(16, os.cpu_count() or 4)) as ex:
            for log in ex.map(_run, jobs_list):
                logs.append(log)
    objs = [OBJ / (s.stem + ".o") for s in cus] + [OBJ / (s.stem + ".cpp.o") for s in cpps]
    lib = LIB / LIBNAME
    if _stale(lib, objs):
        logs.append(_run([nvcc, "-shared", "-gencode", "arch=compute_103a,code=sm_103a",
                          *map(str, objs), "-o", str(lib), "-lpthread"]))
    # host C++ over the C ABI: the Kmeans class library and the gpukmeans CLI
    host_hdrs = sorted(inc.glob("*.hpp")) + sorted(inc.glob("*.h"))
    host_srcs = [s for s in sorted(HOST.glob("*.cpp")) if s.name != "gpukmeans.cpp"]
    hostlib = LIB / "libkmeans_host.so"
    if host_srcs and _stale(hostlib, host_srcs + [lib] + host_hdrs):
        logs.append(_run(["g++", *CXX_FLAGS, "-shared", "-I", str(inc), *map(str, host_srcs),
                          "-o", str(hostlib), "-L", str(LIB), "-lkm_sm103", "-Wl,-rpath,$ORIGIN"]))
    cli = LIB / "gpukmeans"
    if (HOST / "gpukmeans.cpp").exists() and _stale(cli, [HOST / "gpukmeans.cpp", hostlib] + host_hdrs):
        logs.append(_run(["g++", *CXX_FLAGS, "-I", str(inc), str(HOST / "gpukmeans.cpp"),
                          "-o", str(cli), "-L", str(LIB), "-lkmeans_host", "-lkm_sm103",
                          "-Wl,-rpath,$ORIGIN"]))
    if verbose:
        for l in logs:
            if l.strip():
                print(l)
    return lib


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
