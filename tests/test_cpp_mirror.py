"""Builds and runs the C++17 mirror's test program (tests/cpp/test_mirror.cpp)."""
from __future__ import annotations

import subprocess

import pytest

from conftest import ROOT


def _build(wf) -> str:
    out = ROOT / "wavefront-renderer_gb300" / "_build" / "test_mirror"
    out.parent.mkdir(exist_ok=True)
    lib = wf.LIB_PATH
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", str(ROOT / "include"), str(ROOT / "tests" / "cpp" / "test_mirror.cpp"),
                    "-o", str(out), str(lib), f"-Wl,-rpath,{lib.parent}"], check=True)
    return str(out)


def test_cpp_mirror_compiles(wf):
    _build(wf)


@pytest.mark.gpu
def test_cpp_mirror_runs_on_gpu(wf):
    exe = _build(wf)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
