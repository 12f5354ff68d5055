import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def gi():
    """The CUDA library's binding (built in-tree once per session)."""
    from legitengine_gb300 import build
    build.build()
    from legitengine_gb300 import gi as _gi
    _gi.lib()
    return _gi


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as _o
    _o.lib()
    return _o


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def rel_err(a, b, floor=1e-6):
    """Per-element |a - b| / max(|b|, floor)."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.abs(a - b) / np.maximum(np.abs(b), floor)


@pytest.fixture(scope="session")
def scene_small(gi, oracle):
    """A seeded 16-box room at 128x96 with its fp32 oracle G-buffer, shadow map and direct light."""
    prims = gi.scene_generate(1000, 16, 0)
    cam = gi.camera_spline(1, 3, 64)
    view = gi.view_from_camera(cam, 128, 96)
    light = gi.view_from_camera(gi.scene_light(), 256, 256)
    gb = oracle.gbuffer(view, prims)
    sm = oracle.shadow_map(light, prims)
    direct = oracle.direct_light(view, light, gb, sm)
    return {"prims": prims, "view": view, "light": light, "gb": gb, "shadow": sm, "direct": direct}
