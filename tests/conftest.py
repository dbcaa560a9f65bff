import os
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
sys.path.insert(0, HERE)
sys.path.insert(0, REPO)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); parity tests through the C ABI")


@pytest.fixture(scope="session")
def jsb():
    """The product library, built in-tree if needed (fails loudly when the build fails)."""
    from joltphysics_gb300 import build

    build.build()
    import joltphysics_gb300

    joltphysics_gb300.lib()
    return joltphysics_gb300


@pytest.fixture(scope="session")
def oracle_lib():
    from jsb_testlib import Oracle, build_oracle

    build_oracle()
    return Oracle


def golden_path(name):
    return os.path.join(HERE, "golden", f"{name}.npz")
