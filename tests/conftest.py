"""Shared fixtures. GPU tests are marked `gpu`; everything else runs on CPU."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs through the C ABI)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import build_oracle, pyoracle

    build_oracle.build_oracle()
    return pyoracle


@pytest.fixture(scope="session")
def gpu():
    import strouhal_gb300 as sg

    g = sg.GPU(0)
    yield g
    g.close()
