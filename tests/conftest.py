import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


def load_mesh_fixture(name: str):
    from edgefem_gb300.mesh import TetMesh
    d = np.load(os.path.join(GOLDEN, name))
    return TetMesh(d["node_ids"], d["xyz"], d["tets"], d["tet_phys"], d["tris"], d["tri_phys"])


def published():
    with open(os.path.join(GOLDEN, "published.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def wr90_mesh():
    return load_mesh_fixture("rect_waveguide_mesh.npz")


@pytest.fixture(scope="session")
def cube_mesh():
    return load_mesh_fixture("cube_cavity_mesh.npz")


@pytest.fixture(scope="session")
def gpu():
    import edgefem_gb300 as em
    if em.device_count() < 1:
        pytest.skip("no CUDA device")
    return em
