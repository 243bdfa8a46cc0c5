"""Shared fixtures.  GPU tests are marked ``gpu``; everything else runs on CPU."""
from __future__ import annotations

import importlib.util
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
PKG = ROOT / "gravity-simulator_gb300"
GOLDEN = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 GPU and the built CUDA library")


def _module(name: str):
    key = f"gsgpu_{name}"
    if key in sys.modules:
        return sys.modules[key]
    spec = importlib.util.spec_from_file_location(key, PKG / f"{name}.py")
    mod = importlib.util.module_from_spec(spec)
    sys.modules[key] = mod
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="session")
def g():
    """The ctypes mirror of grav_sim's interface (package gsgpu.py)."""
    return _module("gsgpu")


@pytest.fixture(scope="session")
def wl():
    return _module("workloads")


@pytest.fixture(scope="session")
def orc():
    from oracle import restatement
    restatement.load()
    return restatement


@pytest.fixture(scope="session")
def lib(g):
    """The product library.  GPU tests fail loudly if it is missing."""
    return g.load_c_lib()


def golden(name: str):
    with np.load(GOLDEN / f"{name}.npz") as f:
        return {k: f[k] for k in f.files}


def cases(d: dict):
    """Group 'case/key' entries of a golden file by case."""
    out: dict = {}
    for k, v in d.items():
        if "/" in k:
            c, f = k.split("/", 1)
            out.setdefault(c, {})[f] = v
    return out
