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


def _state(C, device, rows=None):
    shape = (C,) if rows is None else (rows, C)  # reward mode keeps per-image rows
    return dict(tp=torch.zeros(shape, dtype=torch.int64, device=device),
                fp=torch.zeros(shape, dtype=torch.int64, device=device),
                fn=torch.zeros(shape, dtype=torch.int64, device=device),
                iou_sum=torch.zeros(shape, dtype=torch.float64, device=device),
                confusion=torch.zeros((C, C + 1), dtype=torch.int64, device=device))


@pytest.mark.parametrize("validate,reward", [(1, 0), (0, 0), (0, 1), (1, 1)])
def test_noalloc_update_matches_update_on_two_calls(validate, reward):
    """Two calls in a row on one stream with no synchronisation between them, then one comparison.

    With validate=0 nothing waits on the host: the second call's clearing of
    the shared array is queued behind the first call's kernels on the same
    stream, which is the only ordering the entry point relies on.
    """
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
    rows = B if reward else None
    with_scratch, no_alloc = _state(C, dev, rows), _state(C, dev, rows)
    pairs = torch.empty((B, G, P), dtype=torch.int64, device=dev)
    areas = torch.empty((B, G + P), dtype=torch.int64, device=dev)
    matched = torch.empty((B, G), dtype=torch.int32, device=dev)
    error = torch.zeros(1, dtype=torch.int32, device=dev)
    s = with_scratch
    for call in range(2):
        assert lib.pe_update(N.ptr(gt), 0, N.ptr(pred), 0, B, pixels, N.ptr(gc), N.ptr(pc), N.ptr(crowd), G, P, C,
                             N.ptr(pairs), N.ptr(areas), N.ptr(matched), N.ptr(s["tp"]), N.ptr(s["fp"]),
                             N.ptr(s["fn"]), N.ptr(s["iou_sum"]), N.ptr(s["confusion"]), None, None, None, None,
                             N.ptr(error), validate, reward, stream) == 0
    torch.cuda.synchronize()
    expected = {key: value.clone() for key, value in with_scratch.items()}
    s = no_alloc
    for call in range(2):
        status = lib.pe_update_noalloc(N.ptr(gt), 0, N.ptr(pred), 0, B, pixels, N.ptr(gc), N.ptr(pc), N.ptr(crowd),
                                       G, P, C, N.ptr(s["tp"]), N.ptr(s["fp"]), N.ptr(s["fn"]), N.ptr(s["iou_sum"]),
                                       N.ptr(s["confusion"]), None, None, None, None, validate, reward, stream)
        assert status == 0, lib.pe_last_error().decode()
    torch.cuda.synchronize()
    for key in ("tp", "fp", "fn", "confusion"):
        assert torch.equal(no_alloc[key], expected[key]), key
    torch.testing.assert_close(no_alloc["iou_sum"], expected["iou_sum"], rtol=RTOL, atol=ATOL)
    assert int(no_alloc["tp"].sum()) > 0


def test_noalloc_rejects_scratch_beyond_its_limit():
    from panoptic_evaluator_gb300 import _native as N
    lib = N.library()
    # 64 x 128 x 128 pairs need 8 MiB of histogram alone: beyond the fixed array.
    status = lib.pe_update_noalloc(None, 0, None, 0, 64, 16, None, None, None, 128, 128, 5, None, None, None, None,
                                   None, None, None, None, None, 0, 0, None)
    assert status == -1
    assert "limit" in lib.pe_last_error().decode()
    # Sizes whose byte counts would wrap a 64-bit integer are rejected before any arithmetic on them.
    for B, G, P in ((2**62, 1, 1), (1, 2**31 - 2, 2**31 - 2), (2**40, 2**20, 2**20)):
        status = lib.pe_update_noalloc(None, 0, None, 0, B, 16, None, None, None, G, P, 5, None, None, None, None,
                                       None, None, None, None, None, 0, 0, None)
        assert status == -1, (B, G, P)
        assert "limit" in lib.pe_last_error().decode()
