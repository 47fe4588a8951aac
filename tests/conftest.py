"""Shared test configuration.

Markers: ``gpu`` — needs a CUDA device and the built ``libgbtomo.so``; everything else
runs on the CPU (oracle vs golden fixtures, host logic, library exports).
"""
from __future__ import annotations

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and libgbtomo.so")


def golden(name: str):
    return np.load(os.path.join(GOLDEN, f"{name}.npz"))


def rel_l2(a, b) -> float:
    a = np.asarray(a, dtype=np.float64).ravel()
    b = np.asarray(b, dtype=np.float64).ravel()
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))


def order_of(variant: str) -> str:
    return "".join({"att": "a", "psf": "p", "psf1d": "p"}[t] for t in variant.split("+")
                   if t != "none")


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pytomography_gb300 import _lib
    _lib.load()
    return torch.device("cuda")


# Relative L2 errors against the float64 oracle recorded by the full-size parity tests,
# printed in the terminal summary so that every run states them per configuration.
PARITY_REPORT: dict = {}


def report_parity(name: str, value: float) -> None:
    PARITY_REPORT[name] = max(float(value), PARITY_REPORT.get(name, 0.0))


def pytest_terminal_summary(terminalreporter, exitstatus, config):
    if not PARITY_REPORT:
        return
    terminalreporter.section("relative L2 vs the float64 oracle (max over the checked items)")
    for k in sorted(PARITY_REPORT):
        terminalreporter.write_line(f"{k}: {PARITY_REPORT[k]:.3e}")
