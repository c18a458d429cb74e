"""Shared test configuration: the ``gpu`` marker and input helpers."""
import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); parity tests through the C-ABI")


def tape(strings):
    """(uint8 data, uint64 offsets) for a list of bytes."""
    strings = [s if isinstance(s, bytes) else s.encode() for s in strings]
    data = np.frombuffer(b"".join(strings), dtype=np.uint8) if strings else np.zeros(0, dtype=np.uint8)
    offsets = np.zeros(len(strings) + 1, dtype=np.uint64)
    offsets[1:] = np.cumsum([len(s) for s in strings])
    return data, offsets


@pytest.fixture(scope="session")
def port():
    from oracle import oracle
    return oracle.Port()
