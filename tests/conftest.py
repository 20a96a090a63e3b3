import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a library)")


def load_golden(name):
    return dict(np.load(os.path.join(GOLDEN, name)))


def golden_meshes(g):
    out = []
    k = 0
    while f"mesh{k}_pos" in g:
        m = g[f"mesh{k}_model"] if bool(g[f"mesh{k}_has_model"]) else None
        out.append((g[f"mesh{k}_pos"], g[f"mesh{k}_idx"], m))
        k += 1
    return out


@pytest.fixture(scope="session")
def port_lib():
    from oracle import oracle as O

    O.build_port()
    return O


@pytest.fixture(scope="session")
def cuda_lib():
    """The sm_103a library, built if needed, with a usable GPU."""
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from rendu_gb300 import build

    build.build()
    import rendu_gb300

    rendu_gb300.lib()
    return rendu_gb300
