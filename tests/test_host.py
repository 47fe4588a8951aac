"""Host-side logic (no GPU): geometry tables, metadata, library exports."""
import ctypes
import os
import re

import numpy as np
import torch

from conftest import ROOT, golden


def test_rotation_theta_matches_restated_kornia():
    from pytomography_gb300 import geometry
    d = golden("theta")
    for size in (23, 24, 92, 182):
        th = geometry.rotation_theta(torch.tensor(d["angles"]), size).numpy()
        assert np.array_equal(th, d[f"theta_{size}"]), size
        assert np.array_equal(geometry.base_grid(size).numpy(), d[f"lin_{size}"])


def test_psf_taps_bitwise_equal_to_reference_layers():
    from pytomography_gb300.metadata.SPECT import SPECTObjectMeta, SPECTProjMeta, SPECTPSFMeta
    from pytomography_gb300.transforms.SPECT import SPECTPSFTransform
    for case in ("spect_even", "spect_odd"):
        d = golden(case)
        shape = tuple(int(s) for s in d["shape"])
        om = SPECTObjectMeta(list(d["dr"]), shape)
        pm = SPECTProjMeta(shape[1:], list(d["dr"][:2]), list(d["angles"]), radii=list(d["radii"]))
        t = SPECTPSFTransform(SPECTPSFMeta((0.03, 0.11)))
        t.configure(om, pm)
        for r in t.radii_unique:
            wr, wz = t.tables[r]
            key = f"psf_att+psf_r{r:g}"
            assert np.array_equal(wr.numpy(), d[key + "_wr"])
            assert np.array_equal(wz.numpy(), d[key + "_wz"])


def test_pad_helpers():
    from pytomography_gb300 import geometry
    for n in (15, 16, 64, 96, 128, 200):
        p = geometry.compute_pad_size(n)
        assert geometry.compute_pad_size_padded(n + 2 * p) == p


def test_library_builds_and_exports_every_declared_symbol():
    from pytomography_gb300 import build
    lib_path = build.build()
    lib = ctypes.CDLL(lib_path)
    header = open(os.path.join(ROOT, "include", "gbtomo.h")).read()
    names = set(re.findall(r"\b(gb_[a-z0-9_]+)\s*\(", header))
    assert names, "no declarations found"
    for n in sorted(names):
        assert hasattr(lib, n), f"{n} declared in gbtomo.h but not exported"
    from pytomography_gb300 import _lib
    declared = {n for n, _, _ in _lib.SIGNATURES}
    assert declared <= names


def test_no_cpu_path_without_cuda():
    import pytest
    if torch.cuda.is_available():
        pytest.skip("CUDA present")
    from pytomography_gb300.metadata.SPECT import SPECTObjectMeta, SPECTProjMeta
    from pytomography_gb300.projectors.SPECT import SPECTSystemMatrix
    om = SPECTObjectMeta([0.4] * 3, (8, 8, 4))
    pm = SPECTProjMeta((8, 4), [0.4] * 2, [0.0, 90.0])
    with pytest.raises(RuntimeError, match="CUDA"):
        SPECTSystemMatrix([], [], om, pm)
