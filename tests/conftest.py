"""Shared test setup: the `gpu` marker, the built libraries, bitwise comparison helpers."""

import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests" / "golden"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (runs on the GB300 box)")


def has_gpu():
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return os.path.exists("/dev/nvidia0")


def pytest_collection_modifyitems(config, items):
    if has_gpu():
        return
    skip = pytest.mark.skip(reason="no CUDA device here")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


@pytest.fixture(scope="session")
def built():
    """Build the package libraries and the oracle once per session."""
    from oracle.build import build as build_oracle
    from pydyn_gb300.build import build

    build()
    build_oracle()
    return True


@pytest.fixture(scope="session")
def dev(built):
    from pydyn_gb300.device import Device

    d = Device(0)
    yield d
    d.close()


def bits(a):
    return np.ascontiguousarray(a, dtype="<f8").view(np.int64)


def assert_bitwise(got, want, name=""):
    got, want = np.asarray(got, dtype=float), np.asarray(want, dtype=float)
    assert got.shape == want.shape, f"{name}: shape {got.shape} vs {want.shape}"
    diff = bits(got) != bits(want)
    if diff.any():
        idx = tuple(int(i) for i in np.argwhere(diff)[0])
        raise AssertionError(
            f"{name}: {int(diff.sum())} of {diff.size} values differ; first at {idx}: "
            f"{got[idx]!r} vs {want[idx]!r} (max |d| {np.abs(got - want)[diff].max():.3e})"
        )
