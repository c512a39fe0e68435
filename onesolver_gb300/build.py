"""Build the native parts of onesolver_gb300 in-tree.

libonesolver.so: the CUDA kernels (sm_103a) and the C ABI, compiled with nvcc
(one process per translation unit, in parallel) and linked with the host-only
C++ sources (the .qubo parser and writers).

The oracle (oracle/, test infrastructure) has its own Makefile; build_oracle()
runs it.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
HOST = PKG / "host"
APPS = PKG / "apps"
OBJ = PKG / "_build"
LIB = PKG / "lib"
LIBNAME = "libonesolver.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build onesolver_gb300")


def cuda_home() -> Path:
    return Path(nvcc()).resolve().parent.parent


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if proc.returncode != 0:
        raise RuntimeError("command failed:\n" + " ".join(cmd) + "\n" + proc.stdout)


def _needs(target: Path, sources: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(s.stat().st_mtime > t for s in sources)


def _headers() -> list[Path]:
    return (sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.hpp")) +
            sorted((ROOT / "include").rglob("*.h*")))


def build_library(verbose: bool = False, jobs: int | None = None) -> Path:
    """Compile every CUDA and host translation unit and link libonesolver.so."""
    OBJ.mkdir(exist_ok=True)
    LIB.mkdir(exist_ok=True)
    inc = ["-I", str(ROOT / "include"), "-I", str(CSRC)]
    common = ["-std=c++17", "-O3", "-Xcompiler", "-fPIC"]
    hdrs = _headers()
    jobs_list = []
    for cu in sorted(CSRC.glob("*.cu")):
        obj = OBJ / (cu.stem + ".o")
        if _needs(obj, [cu, *hdrs]):
            jobs_list.append([nvcc(), *ARCH, "-lineinfo", *common, *inc, "-c", str(cu), "-o", str(obj)])
    for cpp in sorted(HOST.glob("*.cpp")):
        obj = OBJ / (cpp.stem + ".host.o")
        if _needs(obj, [cpp, *hdrs]):
            jobs_list.append(["g++", "-std=c++17", "-O2", "-fPIC", *inc,
                              "-I", str(cuda_home() / "include"), "-c", str(cpp), "-o", str(obj)])
    workers = jobs or max(1, min(len(jobs_list), os.cpu_count() or 4))
    if jobs_list:
        with cf.ThreadPoolExecutor(max_workers=workers) as ex:
            for fut in [ex.submit(_run, c) for c in jobs_list]:
                fut.result()
    objs = sorted(OBJ.glob("*.o"))
    lib = LIB / LIBNAME
    if _needs(lib, objs):
        _run([nvcc(), *ARCH, "-shared", "-o", str(lib), *map(str, objs), "-lcudart"])
    if verbose:
        print(f"built {lib}")
    return lib


def build_apps(verbose: bool = False) -> list[Path]:
    """Build the one-solver-anneal / one-solver-exhaustive CLIs."""
    lib = build_library(verbose=verbose)
    out = []
    for src in sorted(APPS.glob("*.cpp")):
        exe = LIB / src.stem
        if _needs(exe, [src, lib, *_headers()]):
            _run(["g++", "-std=c++17", "-O2", "-I", str(ROOT / "include"), str(src), "-o", str(exe),
                  "-L", str(LIB), "-lonesolver", "-Wl,-rpath,$ORIGIN"])
        out.append(exe)
    return out


def build_oracle(verbose: bool = False) -> Path:
    """Build the CPU oracle (test infrastructure) with its Makefile."""
    _run(["make", "-s", "-C", str(ROOT / "oracle")])
    so = ROOT / "oracle" / "_build" / "liboracle.so"
    if verbose:
        print(f"built {so}")
    return so


if __name__ == "__main__":
    build_library(verbose=True)
    build_apps(verbose=True)
    build_oracle(verbose=True)
    sys.exit(0)
