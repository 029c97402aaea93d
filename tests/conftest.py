"""Test configuration: the `gpu` marker and import paths.

`-m "not gpu"` tests run without a GPU (oracle vs golden vectors, scene compiler, host logic, the
C-ABI's exported symbols and its validation paths); `-m gpu` tests call the CUDA core through
the C-ABI and compare it with the oracle.
"""
import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
for p in (str(ROOT / "dayflower-path-tracer_gb300"), str(ROOT)):
    if p not in sys.path:
        sys.path.insert(0, p)


def reference_resources():
    """The reference checkout's `resources/distribution/resources` directory (models, textures),
    named by the DFPT_REFERENCE_RESOURCES environment variable; None when it is unset or absent.
    Tests that read the reference's own resource files skip without it."""
    v = os.environ.get("DFPT_REFERENCE_RESOURCES")
    if not v:
        return None
    p = Path(v)
    return p if p.is_dir() else None


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libdfpt.so")


@pytest.fixture(scope="session")
def lib():
    from dfpt import _lib

    return _lib.load()


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle

    oracle.load()
    return oracle
