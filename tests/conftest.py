import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "yoxel-voxel_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def _ensure_built():
    import importlib.util
    spec = importlib.util.spec_from_file_location("_yoxel_build", os.path.join(PKG, "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.build()


_ensure_built()


def camera_for(scene_center=(0.5, 0.5, 0.5), direction=(1.0, 0.7, 0.5), dist=1.5):
    """The configs' camera: centre + dist*normalize(direction), looking at the
    centre, up (0,0,1)."""
    c = np.asarray(scene_center, np.float64)
    d = np.asarray(direction, np.float64)
    d = d / np.linalg.norm(d)
    pos = (c + dist * d).astype(np.float32)
    view = (-d).astype(np.float32)
    return pos, view


LIGHT = (np.array([0.3, 0.5, 0.8]) / np.linalg.norm([0.3, 0.5, 0.8])).astype(np.float32)


@pytest.fixture(scope="session")
def oracle():
    from oracle import pyoracle
    pyoracle.lib()
    return pyoracle


@pytest.fixture(scope="session")
def yoxel_mod():
    import yoxel
    return yoxel


def gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
