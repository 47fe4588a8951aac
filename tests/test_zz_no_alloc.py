"""The allocation-free forward projector (collected last on purpose).

``gb_spect_forward_static`` serves callers that cannot allocate device memory while they
run (code on a stream whose memory pool forbids new allocations, hosts whose device memory
belongs to another framework's allocator, services that budget every allocation up
front): its partial sums live in a fixed device array inside the library.
Its output must equal the regular forward projector's, within the 1e-5 relative L2 used
by every parity test, on two calls in a row (the array keeps the previous call's contents).
"""
import ctypes

import numpy as np
import pytest
import torch

from conftest import golden, rel_l2

pytestmark = pytest.mark.gpu


def _static_fn(lib):
    fn = lib.gb_spect_forward_static
    fn.restype = ctypes.c_int32
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32,
                   ctypes.c_void_p]
    return fn


@pytest.mark.parametrize("variant", ["att+psf", "att"])
def test_static_forward_matches_forward_twice(variant, cuda):
    from pytomography_gb300 import _lib
    from pytomography_gb300.metadata.SPECT import SPECTObjectMeta, SPECTProjMeta, SPECTPSFMeta
    from pytomography_gb300.projectors.SPECT import SPECTSystemMatrix
    from pytomography_gb300.transforms.SPECT import SPECTAttenuationTransform, SPECTPSFTransform
    d = golden("spect_even")
    shape = tuple(int(s) for s in d["shape"])
    om = SPECTObjectMeta([float(x) for x in d["dr"]], shape)
    pm = SPECTProjMeta(shape[1:], [float(x) for x in d["dr"][:2]],
                       [float(a) for a in d["angles"]], radii=[float(r) for r in d["radii"]])
    ts = [SPECTAttenuationTransform(torch.tensor(d["mu"], dtype=torch.float32))]
    if "psf" in variant:
        ts.append(SPECTPSFTransform(SPECTPSFMeta((0.03, 0.11))))
    H = SPECTSystemMatrix(ts, [], om, pm)
    H.set_n_subsets(2)
    fn = _static_fn(H._lib)
    f = torch.tensor(d["object"], dtype=torch.float32, device=cuda)
    for subset in (-1, 1):
        ref = H.forward(f, None if subset < 0 else subset)
        for _ in range(2):
            out = torch.full_like(ref, float("nan"))
            _lib.check(fn(H._plan, _lib.ptr(f), _lib.ptr(out), subset, _lib.stream_handle(cuda)))
            torch.cuda.synchronize()
            assert torch.isfinite(out).all()
            assert rel_l2(out.cpu().numpy(), ref.cpu().numpy()) < 1e-5
    assert rel_l2(H.forward(f).cpu().numpy(), d[f"fwd_{variant}_f32"]) < 1e-5


def test_static_forward_rejects_oversized_request(cuda):
    from pytomography_gb300 import _lib
    from pytomography_gb300.metadata.SPECT import SPECTObjectMeta, SPECTProjMeta
    from pytomography_gb300.projectors.SPECT import SPECTSystemMatrix
    n, nz, n_angles = 128, 128, 260  # 260 * 128 * 128 floats > 4,194,304
    om = SPECTObjectMeta([0.4] * 3, (n, n, nz))
    pm = SPECTProjMeta((n, nz), [0.4] * 2, list(np.linspace(0, 360, n_angles, endpoint=False)))
    H = SPECTSystemMatrix([], [], om, pm)
    fn = _static_fn(H._lib)
    f = torch.ones((n, n, nz), device=cuda)
    out = torch.empty((n_angles, n, nz), device=cuda)
    rc = fn(H._plan, _lib.ptr(f), _lib.ptr(out), -1, _lib.stream_handle(cuda))
    assert rc == -2
    assert b"static array" in H._lib.gb_last_error()


def test_static_forward_full_size_subset_and_tuned_plan(cuda):
    """The 128^3 / 120-angle attenuation + PSF workload, one 12-angle subset (about 2.5M
    partial floats, near the 4,194,304 limit), twice in a row; then a tuning with two work
    items per CTA slot, which doubles the partials: rejected at 128^3, accepted (and equal to
    the regular forward) at 16^3."""
    from pytomography_gb300 import _lib, synthetic
    w = synthetic.config2()
    H = synthetic.build_system_matrix(w)
    H.set_n_subsets(10)
    fn = _static_fn(H._lib)
    f = torch.tensor(w.activity, dtype=torch.float32, device=cuda)
    ref = H.forward(f, 4)
    for _ in range(2):
        out = torch.full_like(ref, float("nan"))
        _lib.check(fn(H._plan, _lib.ptr(f), _lib.ptr(out), 4, _lib.stream_handle(cuda)))
        torch.cuda.synchronize()
        assert rel_l2(out.cpu().numpy(), ref.cpu().numpy()) < 1e-5
    H.set_tuning(fwd_items=2)
    out = torch.empty_like(ref)
    assert fn(H._plan, _lib.ptr(f), _lib.ptr(out), 4, _lib.stream_handle(cuda)) == -2
    assert b"static array" in H._lib.gb_last_error()
    # a small plan with the same tuning fits
    from pytomography_gb300.metadata.SPECT import SPECTObjectMeta, SPECTProjMeta, SPECTPSFMeta
    from pytomography_gb300.projectors.SPECT import SPECTSystemMatrix
    from pytomography_gb300.transforms.SPECT import SPECTAttenuationTransform, SPECTPSFTransform
    d = golden("spect_even")
    shape = tuple(int(s) for s in d["shape"])
    om = SPECTObjectMeta([float(x) for x in d["dr"]], shape)
    pm = SPECTProjMeta(shape[1:], [float(x) for x in d["dr"][:2]],
                       [float(a) for a in d["angles"]], radii=[float(r) for r in d["radii"]])
    Hs = SPECTSystemMatrix([SPECTAttenuationTransform(torch.tensor(d["mu"], dtype=torch.float32)),
                            SPECTPSFTransform(SPECTPSFMeta((0.03, 0.11)))], [], om, pm)
    Hs.set_tuning(fwd_items=2)
    fs = torch.tensor(d["object"], dtype=torch.float32, device=cuda)
    ref = Hs.forward(fs)
    for _ in range(2):
        out = torch.full_like(ref, float("nan"))
        _lib.check(fn(Hs._plan, _lib.ptr(fs), _lib.ptr(out), -1, _lib.stream_handle(cuda)))
        torch.cuda.synchronize()
        assert rel_l2(out.cpu().numpy(), ref.cpu().numpy()) < 1e-5
