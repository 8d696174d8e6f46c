"""Shared set-up of the test suite.

Markers: `gpu` — needs a CUDA device (run with -m gpu on a GB300); everything else runs on CPU.
The oracle port is compiled once per session (make -C oracle port, a second); the CUDA extension
is compiled by raw-physics_gb300/build.py when missing or stale (nvcc cross-compiles without a GPU).
"""
from __future__ import annotations

import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "raw-physics_gb300")
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (PKG, ROOT, os.path.join(ROOT, "tests", "golden")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: test needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session")
def oracle_built():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "port"], check=True)
    from oracle.oracle import Oracle
    return Oracle


@pytest.fixture(scope="session")
def ext_built():
    sys.path.insert(0, PKG)
    import build as ext_build
    ext_build.build()
    import rawphys
    rawphys.load_library()
    return rawphys


def golden(name: str):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def scene_fingerprint_ok(scene, g) -> bool:
    """True when this machine's scene generator reproduces the scene the fixture was made from
    (numpy's Generator methods carry no cross-version stream guarantee)."""
    st = g["states"][0] if g["states"].ndim == 3 else g["states"]
    return np.array_equal(st[:, 0:3], scene.pos) and np.array_equal(st[:, 3:7], scene.rot) and \
        np.array_equal(g["invm"][~scene.fixed], 1.0 / scene.mass[~scene.fixed])
