"""Shared test setup: the gpu marker, in-tree builds and package import.

The package directory is named nalu-wind_gb300 (not an identifier), so it is
imported here under the module name nalu_wind_gb300.
"""
from __future__ import annotations

import importlib.util
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


def load_package():
    if "nalu_wind_gb300" in sys.modules:
        return sys.modules["nalu_wind_gb300"]
    pkg_dir = ROOT / "nalu-wind_gb300"
    spec = importlib.util.spec_from_file_location(
        "nalu_wind_gb300", pkg_dir / "__init__.py", submodule_search_locations=[str(pkg_dir)])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["nalu_wind_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


def _build_all():
    sys.path.insert(0, str(ROOT / "nalu-wind_gb300"))
    import build as pkg_build  # nalu-wind_gb300/build.py
    sys.path.pop(0)
    pkg_build.build()
    from oracle import build as ob
    ob.build()


_build_all()


@pytest.fixture(scope="session")
def nw():
    return load_package()


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle
    return oracle


@pytest.fixture(scope="session")
def golds():
    import json
    return json.loads((ROOT / "tests" / "golden" / "reference_golds.json").read_text())


def pytest_sessionfinish(session, exitstatus):
    """With NW_PARITY_REPORT set, write the per-check parity statistics of
    the assembly comparisons (tests/gpu_util.py) to that JSON file."""
    import json
    import os
    path = os.environ.get("NW_PARITY_REPORT")
    if not path:
        return
    gu = sys.modules.get("gpu_util")
    if gu is None:
        return
    Path(path).write_text(json.dumps(gu.PARITY_STATS, indent=1))
