"""Build libnw_gb300.so in-tree for sm_103a (nvcc + g++, no cmake).

Usage: python nalu-wind_gb300/build.py [--force]
Compiles every csrc/*.cu with nvcc (-gencode arch=compute_103a,code=sm_103a)
and every csrc/*.cpp with g++, in parallel, then links one shared library
next to this file. Object files go to _build/ (not committed). Host code is
compiled with -ffp-contract=off, so its floating-point results are the same
on x86_64 and aarch64 hosts (device code uses explicit fma where it fuses).
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
BUILD = PKG / "_build"
LIB = PKG / "libnw_gb300.so"
CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# sources whose device arithmetic must round every multiply and add
# separately (they restate host code compiled with -ffp-contract=off)
NO_FMAD = {"geometry.cu"}


def _nvcc() -> str:
    p = CUDA_HOME / "bin" / "nvcc"
    return str(p) if p.exists() else (shutil.which("nvcc") or "nvcc")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _sources() -> list[Path]:
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))


def _needs_build(force: bool) -> bool:
    if force or not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    deps = _sources() + list(CSRC.glob("*.h")) + list((ROOT / "include").glob("*.h")) + [Path(__file__)]
    return any(p.stat().st_mtime > t for p in deps)


def build(force: bool = False, verbose: bool = False) -> Path:
    if not _needs_build(force):
        return LIB
    BUILD.mkdir(exist_ok=True)
    inc = ["-I", str(ROOT / "include"), "-I", str(CSRC), "-I", str(CUDA_HOME / "include")]
    jobs = []
    for src in _sources():
        obj = BUILD / (src.name + ".o")
        if src.suffix == ".cu":
            cmd = [_nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
                   *(["-fmad=false"] if src.name in NO_FMAD else []),
                   "-Xcompiler", "-fPIC", "-Xcompiler", "-fopenmp", "-Xcompiler", "-ffp-contract=off", *inc, "-c", str(src), "-o", str(obj)]
        else:
            cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", *inc, "-c", str(src), "-o", str(obj)]
        jobs.append((cmd, obj))
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        futs = [ex.submit(_run, c) for c, _ in jobs]
        for f in futs:
            f.result()
    tmp = LIB.with_suffix(".so.tmp")
    link = ["g++", "-shared", "-fopenmp", "-o", str(tmp), *[str(o) for _, o in jobs],
            "-L", str(CUDA_HOME / "lib64"), "-lcudart_static", "-lrt", "-ldl", "-lpthread"]
    _run(link)
    os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
