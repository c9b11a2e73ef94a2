"""Shared test setup.

Markers: `gpu` tests need a CUDA device (they exercise libarec_gb300 on the
GPU); everything else runs on the CPU (the oracle, the host data model, the
C-ABI symbol table, multi-process host logic).
"""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
os.environ.setdefault("ARECGB_QUIET", "1")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built libarec_gb300.so")


@pytest.fixture(scope="session")
def oc():
    import oracle

    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def gb():
    """The CUDA library (built if needed); GPU tests only."""
    import torch

    if not torch.cuda.is_available():
        pytest.fail("gpu test without a CUDA device")
    import arec3d_gb300

    arec3d_gb300.build()
    arec3d_gb300.lib()
    return arec3d_gb300


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    d = np.linalg.norm((a - b).ravel())
    n = np.linalg.norm(b.ravel())
    return d / n if n > 0 else d


def uniform_angles(na, span=np.pi):
    return (np.arange(na) * (span / na)).astype(np.float32)
