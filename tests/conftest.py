"""Test configuration: the `gpu` marker and import paths.

`-m "not gpu"` runs the oracle checks, the host logic and the ABI/export
checks on a machine without a GPU; `-m gpu` runs the parity tests of the CUDA
path against the oracle.
"""

import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "bachelor-thesis_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "tests"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the CUDA path)")


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle

    oracle.build_oracle(ref=True)
    return oracle


@pytest.fixture(scope="session")
def fmlib():
    """The CUDA library, built in-tree for sm_103a."""
    import build as fm_build

    fm_build.build()
    import fluidmarch

    return fluidmarch


@pytest.fixture(scope="session")
def ctx(fmlib):
    c = fmlib.Context(0)
    yield c
    c.close()
