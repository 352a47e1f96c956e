"""Shared pytest setup.

`-m "not gpu"` runs here without a GPU: the oracle against the reference's
pins, host logic and the C-ABI surface. `-m gpu` tests are the parity tests
proper: they call libsed through its C ABI on a GB300 and compare with the
oracle.
"""
import json
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "spin-ed_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs libsed kernels)")


@pytest.fixture(scope="session")
def oracle():
    import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def sed():
    """libsed through its ctypes mirror; builds it when stale."""
    import build_lib
    build_lib.build()
    from spined import internal
    internal.L.load()
    return internal


@pytest.fixture(scope="session")
def pins():
    with open(os.path.join(ROOT, "tests", "golden", "reference_pins.json")) as f:
        return {p["id"]: p for p in json.load(f)["pins"]}
