"""Build the CPU oracle (test infrastructure only): oracle/liboracle.so.

g++ -O3 -ffp-contract=off -fopenmp: no FMA contraction, so the oracle gives
the same FP64 results on x86_64 and aarch64 hosts.
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"


def build(force: bool = False) -> Path:
    src = [HERE / "oracle.cpp", HERE / "gpu_order.cpp", HERE / "oracle.h", Path(__file__)]
    if not force and LIB.exists() and all(p.stat().st_mtime <= LIB.stat().st_mtime for p in src):
        return LIB
    tmp = LIB.with_suffix(".so.tmp")
    cmd = ["g++", "-O3", "-ffp-contract=off", "-std=c++17", "-fPIC", "-shared", "-fopenmp",
           "-o", str(tmp), str(HERE / "oracle.cpp"), str(HERE / "gpu_order.cpp")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
