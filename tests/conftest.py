"""Shared fixtures.  GPU tests are marked `gpu`; everything else runs on CPU.

The oracle (oracle/oracle.py) is the checker only: tests compare the CUDA path
(libwfgpu.so through its C ABI) against it and against the committed golden
fixtures made from the reference's own sources (tests/golden/make_golden.py).
"""
from __future__ import annotations

import importlib.util
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT / "oracle"))
GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


def _load(name, path):
    if name in sys.modules:
        return sys.modules[name]
    spec = importlib.util.spec_from_file_location(name, path)
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="session")
def wf():
    mod = _load("wavefront_gb300", ROOT / "wavefront-renderer_gb300" / "__init__.py")
    if not mod.LIB_PATH.exists():
        _load("wavefront_gb300_build", ROOT / "wavefront-renderer_gb300" / "build.py").build()
    mod.load_library()
    return mod


@pytest.fixture(scope="session")
def orc():
    import oracle

    oracle.port_lib()
    return oracle


@pytest.fixture(scope="session")
def ctx(wf):
    c = wf.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="session")
def scene0(wf):
    return wf.HostScene(0)


@pytest.fixture(scope="session")
def scene_small(wf):
    return wf.HostScene(100, seed=3)


def rays_in_box(rng, n, lo, hi):
    """Random rays from points inside an axis box, directions uniform on the sphere."""
    o = rng.uniform(lo, hi, size=(n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return o, d.astype(np.float32)
