"""Failure detection on the GPU without a fault: injected launch failures come back as
GB_ERR_CUDA and leave the plan usable; a bounded device wait that runs out (its copy is
never issued, so nothing is in flight) returns with the plan's error word set, and the
Python call raises."""
import ctypes

import numpy as np
import pytest
import torch

from conftest import golden, rel_l2

pytestmark = pytest.mark.gpu


def _sm(cuda, **kw):
    from pytomography_gb300.metadata.SPECT import SPECTObjectMeta, SPECTProjMeta, SPECTPSFMeta
    from pytomography_gb300.projectors.SPECT import SPECTSystemMatrix
    from pytomography_gb300.transforms.SPECT import SPECTAttenuationTransform, SPECTPSFTransform
    d = golden("spect_even")
    shape = tuple(int(s) for s in d["shape"])
    om = SPECTObjectMeta([float(x) for x in d["dr"]], shape)
    pm = SPECTProjMeta(shape[1:], [float(x) for x in d["dr"][:2]],
                       [float(a) for a in d["angles"]], radii=[float(r) for r in d["radii"]])
    H = SPECTSystemMatrix([SPECTAttenuationTransform(torch.tensor(d["mu"], dtype=torch.float32)),
                           SPECTPSFTransform(SPECTPSFMeta((0.03, 0.11)))], [], om, pm, **kw)
    return d, H, torch.tensor(d["object"], dtype=torch.float32, device=cuda)


def test_injected_launch_failure_then_recovery(cuda):
    d, H, f = _sm(cuda)
    assert H._lib.gb_inject_fault(b"launch", 1) == 0
    with pytest.raises(RuntimeError, match="injected launch failure"):
        H.forward(f)
    out = H.forward(f)  # fired once: the plan still works
    assert rel_l2(out.cpu().numpy(), d["fwd_att+psf_f32"]) < 1e-5


def test_injected_allocation_failure_on_gpu(cuda):
    from pytomography_gb300 import _lib
    assert _lib.load().gb_inject_fault(b"alloc", 2) == 0
    with pytest.raises(RuntimeError, match="out of memory"):
        _sm(cuda)
    d, H, f = _sm(cuda)
    assert rel_l2(H.forward(f).cpu().numpy(), d["fwd_att+psf_f32"]) < 1e-5


def test_bounded_wait_runs_out_and_reports(cuda):
    d, H, f = _sm(cuda, check_device_status=True)
    H.set_tuning(fwd_variant=1)  # the forward with TMA attenuation copies and bounded waits
    assert H.device_status() == 0
    # every work item's first attenuation copy is left unissued; each wait gives up after
    # 16 polls of at most 20 us
    assert H._lib.gb_spect_set_debug(H._plan, 1, 16) == 0
    with pytest.raises(RuntimeError, match="gave up waiting"):
        H.forward(f)
    torch.cuda.synchronize()  # the context is still usable
    assert H.device_status() == 0  # raising reset the word
    assert H._lib.gb_spect_set_debug(H._plan, 0, 0) == 0
    out = H.forward(f)
    assert H.device_status() == 0
    assert rel_l2(out.cpu().numpy(), d["fwd_att+psf_f32"]) < 1e-5


def test_pool_memory_release_keeps_live_plans_usable(cuda):
    """Destroyed plans' blocks go back to the driver; a live plan still projects correctly
    and a new plan can be built afterwards."""
    import gc
    import pytomography_gb300 as p
    d, H, f = _sm(cuda)
    ref = H.forward(f)
    _, H2, _ = _sm(cuda)
    del H2
    gc.collect()
    p.release_pool_memory()
    assert torch.equal(H.forward(f), ref)
    _, H3, _ = _sm(cuda)
    assert torch.equal(H3.forward(f), ref)


def test_plan_churn_reuses_pool_memory(cuda):
    """Creating and destroying the same plan repeatedly reuses the pool's blocks: after the
    first round the device's free memory does not shrink further."""
    import gc
    torch.cuda.synchronize()
    free = []
    for _ in range(6):
        d, H, f = _sm(cuda)
        H.forward(f)
        del H
        gc.collect()
        torch.cuda.synchronize()
        free.append(torch.cuda.mem_get_info()[0])
    assert min(free[1:]) >= free[0] - (64 << 20), free
