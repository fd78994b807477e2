"""Pointer arithmetic of the host paths, checked on CPU tensors with the native call captured (no GPU work).

The prefix and panoptic-compute paths pass the kernels pointers computed from
one or two allocations instead of tensor views; these tests hold every pointer
against the view that the results expose for the same field.
"""

import contextlib
import ctypes

import numpy as np
import pytest
import torch

from panoptic_evaluator_gb300 import _native as N


@pytest.fixture
def captured(monkeypatch):
    calls = []
    monkeypatch.setattr(N, "call", lambda name, *args: calls.append((name, args)) or 0)
    monkeypatch.setattr(N, "stream_handle", lambda device=None: 0)
    monkeypatch.setattr(N, "on_device", lambda device: contextlib.nullcontext())
    empty = torch.empty
    monkeypatch.setattr(torch, "empty", lambda *a, pin_memory=False, **k: empty(*a, **k))
    return calls


def test_compute_one_pointers_address_the_returned_views(captured):
    from panoptic_evaluator_gb300._cuda_evaluator import compute_one
    C = 7
    state = [torch.zeros(C, dtype=torch.int64) for _ in range(3)] + [torch.zeros(C, dtype=torch.float64),
                                                                     torch.zeros((C, C + 1), dtype=torch.int64),
                                                                     torch.ones(C, dtype=torch.bool)]
    rows, summaries, counts, miou, copies = compute_one(*state, C)
    (name, args), = captured
    assert name == "pe_compute" and args[6:8] == (1, C)
    expected = [rows[0], summaries[0], counts[0], miou, *copies]  # per_class, summaries, counts, miou, snapshots
    assert list(args[8:17]) == [t.data_ptr() for t in expected]
    assert [r.shape for r in rows] == [(C,)] * 4 and len(summaries) == 9 and len(counts) == 3 and miou.dim() == 0
    assert copies[4].shape == (C, C + 1) and copies[4].data_ptr() % 16 == 0  # copied in 16-byte words
    # pq, sq, rq and IoU rows are adjacent: the kernel writes them as one [4, C] block.
    assert [r.data_ptr() - rows[0].data_ptr() for r in rows] == [0, 8 * C, 16 * C, 24 * C]


def _prefix_inputs(B=3, H=6, W=5, S=4):
    from panoptic_evaluator_gb300 import prefix as PF
    rng = np.random.default_rng(0)
    maps = torch.zeros((B, H, W), dtype=torch.int32)
    gc = torch.zeros((B, S), dtype=torch.int32)
    crowd = torch.zeros((B, S), dtype=torch.bool)
    n = [2, 0, 5][:B]
    masks = [torch.from_numpy(rng.random((k, H, W)) < 0.5) for k in n]
    classes = [torch.arange(k, dtype=torch.int32) for k in n]
    points = [[0, 1, 2], [0], [1, 3, 5]][:B]
    return PF, maps, gc, crowd, masks, classes, points


def test_prefix_pointers_address_the_outputs_and_tables(captured):
    PF, maps, gc, crowd, masks, classes, points = _prefix_inputs()
    things = torch.ones(11, dtype=torch.uint8)
    thresholds = (0.5, 0.75)
    out, rows, _, thr = PF.run_prefixes(maps, gc, crowd, masks, classes, 11, things, thresholds, points, False)
    (name, args), = captured
    assert name == "pe_prefix"
    B, S, T, C, R = 3, 4, 2, 11, sum(map(len, points))
    assert args[1] == B and args[3] == R and args[4] == S and args[13:15] == (T, C)
    keys = ("tp", "fp", "fn", "sums", "confusion", "itp", "ifp", "ifn", "precision", "recall", "values",
            "summaries", "counts", "miou")
    assert list(args[23:37]) == [out[k].data_ptr() for k in keys]
    shapes = {"tp": (R, C), "confusion": (R, C, C + 1), "itp": (R, T, C), "values": (R, 4, C),
              "summaries": (R, 3, 3), "counts": (R, 3), "miou": (R,)}
    for key, shape in shapes.items():
        assert tuple(out[key].shape) == shape
    assert out["sums"].dtype == torch.float64 and out["tp"].dtype == torch.int64
    # Fields are laid out one after another, then the chunk counter of the owner pass.
    ends = [out[k].data_ptr() + 8 * out[k].numel() for k in keys]
    assert ends[:-1] == [out[k].data_ptr() for k in keys[1:]] and args[39] == ends[-1]
    # Thresholds, descriptors and the step table travel in one upload, read back through the pointers.
    assert args[12] == thr.data_ptr() and list(thr) == list(thresholds)
    desc = np.ctypeslib.as_array((ctypes.c_int64 * (B * PF.FIELDS)).from_address(args[0])).reshape(B, PF.FIELDS)
    assert list(desc[:, PF.NMASK]) == [2, 0, 5] and list(desc[:, PF.NQ]) == [3, 1, 3]
    steps = np.ctypeslib.as_array((ctypes.c_int32 * int(sum(k + 1 for k in (2, 0, 5)))).from_address(args[7]))
    want = np.full(steps.size, -1)
    for b, (begin, pts) in enumerate(zip(desc[:, PF.STEP_BEGIN], points)):
        for i, k in enumerate(pts):
            want[begin + k] = i
    assert list(steps) == list(want)
    # int32 workspaces back to back: ga [B x S], raw, pairs, counters [B x T x C x 2], error.
    raw_len, pairs_len = args[18], args[20]
    assert args[16] == B * S and args[22] == B * T * C * 2 and raw_len == S * 7
    assert args[17] - args[15] == 4 * B * S and args[19] - args[17] == 4 * max(raw_len, 1)
    assert args[21] - args[19] == 4 * max(pairs_len, 1) and args[40] - args[21] == 4 * B * T * C * 2
    assert list(rows) == [0, 3, 4]


def test_prefix_checkpoint_tables_match_for_shared_and_distinct_checkpoints(captured):
    PF, maps, gc, crowd, masks, classes, _ = _prefix_inputs()
    things = torch.ones(11, dtype=torch.uint8)
    tables = []
    for points in ([[0], [0], [0]], [[0], [0], [1]]):  # shared (broadcast table), then distinct
        captured.clear()
        PF.run_prefixes(maps, gc, crowd, masks, classes, 11, things, (0.5,), points, False)
        (_, args), = captured
        tables.append(list(np.ctypeslib.as_array((ctypes.c_int32 * 10).from_address(args[7]))))
    # Images with 2, 0 and 5 masks: prefix slots 3, 1 and 6; checkpoint 0 first, then 1 for the last image.
    assert tables[0] == [0, -1, -1, 0, 0, -1, -1, -1, -1, -1]
    assert tables[1] == [0, -1, -1, 0, -1, 0, -1, -1, -1, -1]
