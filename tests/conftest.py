import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built libgblap.so")


@pytest.fixture(scope="session")
def golden():
    return np.load(os.path.join(ROOT, "tests", "golden", "golden.npz"))


GOLDEN_CASES = ["grid2d", "grid3d", "chunglu", "knn", "aniso"]
GOLDEN_PRECS = ["line_jacobi", "GS_std", "ichol", "it_jacobi", "GS_it", "GS_it2", "none"]


def golden_matrix(g, name):
    return (int(g[f"{name}_ia"].shape[0] - 1), g[f"{name}_ia"], g[f"{name}_ja"], g[f"{name}_a"],
            g[f"{name}_b"])
