import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = Path(__file__).resolve().parent / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs through the C ABI of libb3gpu.so")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Compile the CUDA library (sm_103a, cross-compiles without a GPU) and the CPU oracle once."""
    from bullet3_gb300 import _build
    from oracle import build as oracle_build
    _build.build_library()
    oracle_build.build_oracle()
    yield


def gpu_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return os.path.exists("/dev/nvidia0")


def load_golden(name):
    import numpy as np
    return dict(np.load(GOLDEN / f"{name}.npz"))


def shapes_from(d):
    from oracle import oracle as O
    return O.Shapes(d["shape_collidables"], d["shape_local_aabbs"], d["shape_hulls"], d["shape_faces"],
                    d["shape_indices"], d["shape_verts"], d["shape_edges"], d.get("shape_children"))
