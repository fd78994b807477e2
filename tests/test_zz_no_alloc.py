"""pe_update_noalloc: the panoptic update for callers that cannot allocate device memory.

Some host applications cannot call cudaMalloc (their device memory belongs to
another runtime's allocator, or an allocation would synchronise a
latency-critical loop). pe_update_noalloc takes its scratch from a fixed array
inside the library instead of caller buffers. This test calls it through the C
ABI and checks it against pe_update (which receives caller-allocated scratch)
on two calls in a row, within the tolerance of the other GPU tests (integers
exact, FP64 1e-12). The file is named to be collected last.
"""

import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

RTOL = ATOL = 1e-12


def _state(C, device):
    return dict(tp=torch.zeros(C, dtype=torch.int64, device=device),
                fp=torch.zeros(C, dtype=torch.int64, device=device),
                fn=torch.zeros(C, dtype=torch.int64, device=device),
                iou_sum=torch.zeros(C, dtype=torch.float64, device=device),
                confusion=torch.zeros((C, C + 1), dtype=torch.int64, device=device))


def test_noalloc_update_matches_update_on_two_calls():
    from panoptic_evaluator_gb300 import build, synthetic
    from panoptic_evaluator_gb300 import _native as N
    build.build()
    lib = N.library()
    a = synthetic.coco_panoptic_batch(seed=21, B=4, canvas=256, side=(200, 256))
    dev = torch.device("cuda", 0)
    t = lambda x: torch.from_numpy(np.ascontiguousarray(x)).to(dev)  # noqa: E731
    gt, pred, gc, pc, crowd = t(a.gt), t(a.pred), t(a.gc), t(a.pc), t(a.crowd).view(torch.uint8)
    B, G, P, C = gt.shape[0], gc.shape[1], pc.shape[1], a.num_classes
    pixels = gt.shape[1] * gt.shape[2]
    stream = N.stream_handle(dev)
    with_scratch, no_alloc = _state(C, dev), _state(C, dev)
    pairs = torch.empty((B, G, P), dtype=torch.int64, device=dev)
    areas = torch.empty((B, G + P), dtype=torch.int64, device=dev)
    matched = torch.empty((B, G), dtype=torch.int32, device=dev)
    error = torch.zeros(1, dtype=torch.int32, device=dev)
    for call in range(2):
        s = with_scratch
        assert lib.pe_update(N.ptr(gt), 0, N.ptr(pred), 0, B, pixels, N.ptr(gc), N.ptr(pc), N.ptr(crowd), G, P, C,
                             N.ptr(pairs), N.ptr(areas), N.ptr(matched), N.ptr(s["tp"]), N.ptr(s["fp"]),
                             N.ptr(s["fn"]), N.ptr(s["iou_sum"]), N.ptr(s["confusion"]), None, None, None, None,
                             N.ptr(error), 1, 0, stream) == 0
        s = no_alloc
        status = lib.pe_update_noalloc(N.ptr(gt), 0, N.ptr(pred), 0, B, pixels, N.ptr(gc), N.ptr(pc), N.ptr(crowd),
                                       G, P, C, N.ptr(s["tp"]), N.ptr(s["fp"]), N.ptr(s["fn"]), N.ptr(s["iou_sum"]),
                                       N.ptr(s["confusion"]), None, None, None, None, 1, 0, stream)
        assert status == 0, lib.pe_last_error().decode()
        torch.cuda.synchronize()
        for key in ("tp", "fp", "fn", "confusion"):
            assert torch.equal(no_alloc[key], with_scratch[key]), (call, key)
        torch.testing.assert_close(no_alloc["iou_sum"], with_scratch["iou_sum"], rtol=RTOL, atol=ATOL)
    assert int(no_alloc["tp"].sum()) > 0


def test_noalloc_rejects_scratch_beyond_its_limit():
    from panoptic_evaluator_gb300 import _native as N
    lib = N.library()
    # 64 x 128 x 128 pairs need 8 MiB of histogram alone: beyond the fixed array.
    status = lib.pe_update_noalloc(None, 0, None, 0, 64, 16, None, None, None, 128, 128, 5, None, None, None, None,
                                   None, None, None, None, None, 0, 0, None)
    assert status == -1
    assert "limit" in lib.pe_last_error().decode()
