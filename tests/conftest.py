"""Test configuration.

Markers: `gpu` tests need a CUDA device and the built library; everything else
runs on the CPU (oracle known-answer tests, ABI/symbol checks, host logic).
The oracle (oracle/) is the checker only: tests compare the GPU library with it.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built geon_gb300 library")


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle
    oracle.lib()
    return oracle


@pytest.fixture(scope="session")
def geon():
    from geon_gb300 import build
    build.build()
    import geon_gb300
    geon_gb300._load()
    return geon_gb300
