import json
import sys
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parents[1]
PKG_PY = REPO / "aero-cfd-solver_gb300" / "python"
for p in (str(REPO), str(PKG_PY)):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = REPO / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: longer CPU test")


@pytest.fixture(scope="session")
def golden_meshes():
    return np.load(GOLDEN / "meshes.npz")


@pytest.fixture(scope="session")
def golden_residuals():
    data = np.load(GOLDEN / "residuals.npz")
    return data, json.loads(str(data["meta"]))


@pytest.fixture(scope="session")
def golden_histories():
    data = np.load(GOLDEN / "histories.npz")
    return data, json.loads(str(data["meta"]))


def golden_mesh(meshes, name):
    from aero_gb300 import capi

    g = lambda k: meshes[f"{name}/{k}"]  # noqa: E731
    return capi.Mesh(g("owner"), g("neighbor"), g("bc"), g("normal"), g("center"), g("area"),
                     g("volume"), g("cell_center"), g("wall_faces"), points=g("points"),
                     face_vertices=g("face_vertices"), cell_conn=g("cell_conn"))
