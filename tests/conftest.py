"""Shared fixtures. Tests marked `gpu` need a CUDA device and the sm_103a library;
everything else runs on the CPU (oracle pins, host contracts, ABI surface)."""

import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as o

    o.load()
    return o


@pytest.fixture(scope="session")
def device():
    from rohditor_gb300 import Device

    dev = Device(0)
    yield dev
    dev.close()


@pytest.fixture(scope="session")
def stages(device):
    from rohditor_gb300 import Stages

    return Stages(device)
