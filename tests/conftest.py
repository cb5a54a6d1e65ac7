"""Shared test fixtures.

Markers: `gpu` — needs a CUDA GPU (run with -m gpu on a GB300); everything else runs on CPU.
Parity tests record the errors they measure; with SPH_REPORT_DIR set, the records are
written to <dir>/parity_report.json at the end of the session.
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

_REPORT: list[dict] = []


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


def pytest_sessionfinish(session, exitstatus):
    d = os.environ.get("SPH_REPORT_DIR")
    if d and _REPORT:
        os.makedirs(d, exist_ok=True)
        with open(os.path.join(d, "parity_report.json"), "w") as f:
            json.dump(_REPORT, f, indent=1)


@pytest.fixture(scope="session")
def sphlib():
    """The CUDA library (built in-tree if needed; loading needs no GPU)."""
    from tmp_sph_gb300 import build, api
    build.build()
    return api.lib()


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.lib()
    return O


@pytest.fixture
def report(request):
    """report(quantity, value, tol, **extra): record a measured error."""
    def _rec(quantity, value, tol=None, **extra):
        _REPORT.append({"test": request.node.nodeid, "quantity": quantity,
                        "value": float(value), "tol": None if tol is None else float(tol),
                        **extra})
    return _rec


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a CUDA device")
    return torch.device("cuda:0")


def rel_l2(a, b, floor=0.0):
    """||a - b|| / max(||b||, floor)."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    den = max(float(np.linalg.norm(b)), floor)
    if den == 0.0:
        return float(np.linalg.norm(a - b))
    return float(np.linalg.norm(a - b)) / den
