"""Test configuration: the ``gpu`` marker and shared helpers.

CPU tests (``-m "not gpu"``) cover the FP64 oracle against the reference's
golden vectors, host-side logic and that the C-ABI library exports every
symbol of include/seis_gb300.h.  GPU tests (``-m gpu``) are the parity tests:
the CUDA engine, called through the C ABI, against the oracle.
"""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


_PARITY = []


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


def pytest_terminal_summary(terminalreporter):
    """The measured errors of the parity tests, printed whatever the verbosity."""
    if _PARITY:
        terminalreporter.section("parity (relative L2 against the FP64 oracle / the reference)")
        for name, errs in _PARITY:
            terminalreporter.write_line(f"{name}: " + ", ".join(f"{k} {v:.2e}" for k, v in errs.items()))


@pytest.fixture
def parity_report():
    """report(name, **errors): record measured errors for the end-of-run summary."""
    def report(name, **errs):
        _PARITY.append((name, {k: float(v) for k, v in errs.items()}))
    return report


def rel_l2(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def load_golden(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as orc
    orc.set_threads(min(16, os.cpu_count() or 1))
    return orc
