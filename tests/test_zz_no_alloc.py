"""pyrsgm_gb300_compute_level_noalloc against pyrsgm_compute_level.

The no-alloc entry point serves callers that are not allowed to allocate
device memory (hosts that own every byte of it, real-time loops that cannot
afford cudaMalloc's implicit synchronisation).  It must give exactly what the
workspace-based entry point gives -- disparity x16 bit-exact, float
disparity and confidence within 1e-6 absolute -- and what the reference's
own kernels give on the same inputs, on calls in a row that lay the shared
static scratch out differently: a Birchfield-Tomasi coarse level with 64
labels first, then a Census refine level with 16 labels (whose buffers sit
where the first call left its own), then a level close to the scratch limit
(480x360, 16 labels, about 30 MB).  Once every kernel has been loaded, a
further call must leave the device's free memory unchanged.  A level larger
than the scratch is refused before any device work.

This file is collected last so that a run stopping at the first failure has
run every other test already.
"""
from __future__ import annotations

import numpy as np
import pytest

from tests import _oracle, _runners, cases

pytestmark = pytest.mark.gpu

NEAR_LIMIT = cases._lvl("noalloc_census_refine_480x360", 480, 360, 16, cases.CENSUS, True, seed=21)


def _noalloc(case: dict) -> dict:
    import torch
    from pyrsgm_gb300._native import lib
    left, right, (pd, pc) = _runners.inputs(case)
    h, w = left.shape
    L = torch.from_numpy(left).cuda()
    R = torch.from_numpy(right).cuda()
    PD = torch.from_numpy(pd).cuda() if pd is not None else None
    PC = torch.from_numpy(pc).cuda() if pc is not None else None
    ph, pw = pd.shape if pd is not None else (0, 0)
    d16 = torch.zeros((h, w), dtype=torch.int16, device="cuda")
    d32 = torch.zeros((h, w), dtype=torch.float32, device="cuda")
    cf = torch.zeros((h, w), dtype=torch.float32, device="cuda")
    a = case["p2p"]
    rc = lib().pyrsgm_gb300_compute_level_noalloc(
        L.data_ptr(), R.data_ptr(), PD.data_ptr() if PD is not None else None,
        PC.data_ptr() if PC is not None else None, d16.data_ptr(), d32.data_ptr(), cf.data_ptr(),
        w, w, pw * 2, pw * 4, w * 2, w * 4, w * 4, w, h, pw, ph, case["D"], 0, case["maxD"], case["bs"], case["P1"],
        case["P2"], case["uniq"], case["maxdiff"], case["pfc"], case["cost"], case["post"], case["paths"],
        int(case["refine"]), case["minConf"], int(case["adaptive"]), a[0], a[1], a[2], a[3],
        torch.cuda.current_stream().cuda_stream)
    assert rc == 0
    torch.cuda.synchronize()
    return dict(disp16=d16.cpu().numpy(), disp32=d32.cpu().numpy(), conf=cf.cpu().numpy())


def test_noalloc_matches_compute_level_and_reference_on_calls_in_a_row():
    from pyrsgm_gb300._native import lib
    order = (cases.LEVELS[1], cases.LEVELS[4], NEAR_LIMIT)   # BT coarse 64 labels; Census refine; near the limit
    assert lib().pyrsgm_gb300_workspace_bytes(480, 360, 16) <= 32 << 20
    for case in order:
        got = _noalloc(case)
        want = _runners.run_mine(case, with_volumes=False)
        bad = _runners.compare(got, want, volumes=False)
        assert not bad, (case["name"], "vs pyrsgm_compute_level", bad)
        if _oracle.ref_available():
            bad = _runners.compare(got, _runners.run_ref(case), volumes=False)
            assert not bad, (case["name"], "vs reference kernels", bad)
        assert np.sum(got["disp32"] > 0) > 0


def test_noalloc_call_allocates_no_device_memory():
    import torch
    first, second = cases.LEVELS[1], cases.LEVELS[4]
    _noalloc(first)
    _noalloc(second)          # every kernel both layouts need is loaded now
    from pyrsgm_gb300._native import lib
    left, right, (pd, pc) = _runners.inputs(first)
    h, w = left.shape
    L, R = torch.from_numpy(left).cuda(), torch.from_numpy(right).cuda()
    d16 = torch.zeros((h, w), dtype=torch.int16, device="cuda")
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    a = first["p2p"]
    rc = lib().pyrsgm_gb300_compute_level_noalloc(
        L.data_ptr(), R.data_ptr(), None, None, d16.data_ptr(), None, None, w, w, 0, 0, w * 2, 0, 0, w, h, 0, 0,
        first["D"], 0, first["maxD"], first["bs"], first["P1"], first["P2"], first["uniq"], first["maxdiff"],
        first["pfc"], first["cost"], first["post"], first["paths"], 0, first["minConf"], int(first["adaptive"]),
        a[0], a[1], a[2], a[3], torch.cuda.current_stream().cuda_stream)
    assert rc == 0
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0


def test_noalloc_refuses_a_level_larger_than_its_scratch():
    import torch
    from pyrsgm_gb300._native import lib
    img = torch.zeros((16, 16), dtype=torch.uint8, device="cuda")
    out = torch.zeros((16, 16), dtype=torch.int16, device="cuda")
    # 4096 x 2048 with 256 labels needs ~8.6 GB of scratch: rejected before any device work
    rc = lib().pyrsgm_gb300_compute_level_noalloc(
        img.data_ptr(), img.data_ptr(), None, None, out.data_ptr(), None, None, 16, 16, 0, 0, 32, 0, 0,
        4096, 2048, 0, 0, 256, 0, 255, 5, 8, 32, 10, 1, 63, 1, 1, 3, 0, 0.05, 0, 1.0, 1.0, 1.0, 1.0,
        torch.cuda.current_stream().cuda_stream)
    assert rc == -1
    torch.cuda.synchronize()
