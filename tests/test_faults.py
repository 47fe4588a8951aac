"""Failure detection without a GPU fault: the C ABI's host-side fault injector.

Each injected failure must come back as the documented negative status with a message in
gb_last_error(), exactly once, and leave the library usable.  These checks run on the CPU
(the injected sites return before any device work); the GPU variants are in
tests/test_faults_gpu.py.
"""
import ctypes
import os
import subprocess
import sys

import pytest

from conftest import ROOT


@pytest.fixture(scope="module")
def lib():
    from pytomography_gb300 import _lib, build
    build.build()
    lib = ctypes.CDLL(build.LIB)
    for name, res, args in _lib.SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


def test_injected_bad_argument_once(lib):
    assert lib.gb_inject_fault(b"arg", 1) == 0
    rc = lib.gb_spect_forward(None, None, None, -1, None)
    assert rc == -1 and b"injected bad argument" in lib.gb_last_error()
    # the site fired once: the next call reports the real (null-pointer) check
    rc = lib.gb_spect_forward(None, None, None, -1, None)
    assert rc == -1 and b"null argument" in lib.gb_last_error()


def test_injected_allocation_failure_at_plan_creation(lib):
    from pytomography_gb300 import _lib, geometry
    import numpy as np
    import torch
    n, nz = 8, 4
    Lp = n + 2 * geometry.compute_pad_size(n)
    ang = torch.tensor([0.0, 90.0])
    keep = [geometry.rotation_theta(-(270 - ang), Lp).numpy(),
            geometry.rotation_theta(270 - ang, Lp).numpy(), geometry.base_grid(Lp).numpy()]
    d = _lib.SpectDesc()
    d.nx = d.ny = n
    d.nz = nz
    d.dx = d.dy = d.dz = 0.4
    d.n_angles = 2
    d.theta_fwd, d.theta_bwd, d.lin = (k.ctypes.data_as(ctypes.c_void_p) for k in keep)
    d.order = b""
    h = ctypes.c_void_p()
    assert lib.gb_inject_fault(b"alloc", 1) == 0
    rc = lib.gb_spect_plan_create(ctypes.byref(d), ctypes.byref(h))
    assert rc == -3, lib.gb_last_error()
    assert b"out of memory" in lib.gb_last_error()
    assert not h.value
    assert np.isfinite(keep[0]).all()


def test_injector_arms_from_the_environment():
    code = (
        "import ctypes, sys; sys.path.insert(0, %r)\n"
        "from pytomography_gb300 import build\n"
        "lib = ctypes.CDLL(build.LIB)\n"
        "lib.gb_last_error.restype = ctypes.c_char_p\n"
        "f = lib.gb_spect_forward\n"
        "f.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_int32, ctypes.c_void_p]\n"
        "rcs = [f(None, None, None, -1, None) for _ in range(3)]\n"
        "print(rcs, lib.gb_last_error().decode())\n" % ROOT)
    env = dict(os.environ, GBTOMO_INJECT="arg:2")
    out = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True,
                         timeout=120)
    assert out.returncode == 0, out.stderr
    # every call fails the null check; the second one fails at the injected site instead
    assert "[-1, -1, -1]" in out.stdout


def test_unknown_site_is_rejected(lib):
    assert lib.gb_inject_fault(b"disk", 1) == -1
    assert b"unknown fault site" in lib.gb_last_error()
    assert lib.gb_inject_fault(b"arg", 0) == 0
