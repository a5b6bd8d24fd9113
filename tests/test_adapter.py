"""The C++ LinearSystem layer of include/nw_linear_system.hpp (the
reference's LinearSystem::create / PetraType factory, LinearSolverConfig
strings and LinearSystem members over the C ABI), compiled and run as a
nalu-wind build would link it: host checks here, the full assemble + solve
path on the GPU."""
import os
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
CUDA = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))


@pytest.fixture(scope="module")
def adapter_bin(tmp_path_factory, nw):
    nw.load()
    out = tmp_path_factory.mktemp("adapter") / "adapter_check"
    pkg = ROOT / "nalu-wind_gb300"
    cmd = ["g++", "-std=c++17", "-O1", "-I", str(ROOT / "include"), "-I", str(CUDA / "include"),
           str(ROOT / "tests" / "adapter_check.cpp"), "-o", str(out), "-L", str(pkg), "-l:libnw_gb300.so",
           f"-Wl,-rpath,{pkg}", "-L", str(CUDA / "lib64"), "-lcudart", f"-Wl,-rpath,{CUDA / 'lib64'}"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return out


def test_adapter_factory_and_graph_on_the_host(adapter_bin):
    r = subprocess.run([str(adapter_bin), "host"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "host checks passed" in r.stdout


@pytest.mark.gpu
def test_adapter_assemble_and_solve_on_the_gpu(adapter_bin):
    r = subprocess.run([str(adapter_bin), "device"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "device checks passed" in r.stdout
