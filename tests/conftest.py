"""Shared test set-up: import paths, the `gpu` marker, golden fixtures, synthetic systems."""
from __future__ import annotations

import json
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
for p in (ROOT, ROOT / "porousmaterials.jl_gb300", ROOT / "oracle", ROOT / "tests"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))

GOLDEN_DIR = ROOT / "tests" / "golden"
DATA = GOLDEN_DIR / "data"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built libpmgb.so")


@pytest.fixture(scope="session")
def golden():
    return json.loads((GOLDEN_DIR / "golden.json").read_text())


@pytest.fixture(scope="session", autouse=True)
def _data_paths(tmp_path_factory):
    import pmgb

    pmgb.set_paths(DATA)
    # results the drop-ins save (autosave, .cube files) go to the session's temporary folder
    out = tmp_path_factory.mktemp("pm_output")
    pmgb.rc["paths"]["simulations"] = str(out / "simulations")
    pmgb.rc["paths"]["grids"] = str(out / "grids")
    yield


@pytest.fixture(scope="session")
def ref_masses():
    """Atomic masses from the reference's data set (for per-mass unit conversions)."""
    masses = {}
    for line in (DATA / "atomicmasses.csv").read_text().splitlines()[1:]:
        if line.strip():
            k, v = line.split(",")
            masses[k.strip()] = float(v)
    return masses


@pytest.fixture(scope="session")
def ctx():
    import pmgb

    return pmgb.Context.default(0)
