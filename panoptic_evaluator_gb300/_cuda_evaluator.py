"""Drop-in module for the reference's ``panoptic_evaluator._cuda_evaluator``.

It exposes the reference extension's op names and signatures
(panoptic_evaluator/csrc/bindings.cpp:28-57) on top of the pe_gb300 C ABI, so
the reference's own Python layer can import this module in its place. Tensor
checks raise ``RuntimeError`` like the reference's ``TORCH_CHECK``; ops that
allocate in the reference allocate their outputs here with torch, then call
the C ABI on the current stream.
"""

from __future__ import annotations

import torch

from . import _native as N


def _require(condition, message):
    if not condition:
        raise RuntimeError(message)


def _check(tensor, reference, dtype, name="tensor"):
    _require(tensor.device == reference.device and tensor.is_contiguous() and tensor.dtype == dtype,
             f"incorrect {name} device, layout or dtype")


def _lookup(ids, slots, classes, reference):
    _require((ids is None) == (slots is None), "lookup IDs and slots must be supplied together")
    if ids is None:
        return None, None
    _check(ids, reference, torch.int64, "lookup IDs")
    _check(slots, reference, torch.int32, "lookup slots")
    _require(ids.shape == classes.shape and slots.shape == classes.shape, "incorrect lookup shape")
    return ids, slots


def update(gt, pred, gc, pc, crowd, pairs, areas, matched, tp, fp, fn, iou_sum, confusion,
           gt_ids=None, gt_slots=None, pred_ids=None, pred_slots=None, error=None, validate=True, reward=False):
    """Count intersections, validate and accumulate (histogram_kernel.cu:257-341)."""
    _require(gt.is_cuda and gt.dim() == 3, "gt must be CUDA B x H x W")
    for t in (gt, pred):
        _require(t.device == gt.device and t.is_contiguous() and t.dtype in (torch.int32, torch.int64),
                 "maps must be contiguous int32 or int64 on the same CUDA device")
    for t in (gc, pc, matched, error):
        _check(t, gt, torch.int32)
    for t in (pairs, areas, tp, fp, fn, confusion):
        _check(t, gt, torch.int64)
    _check(crowd, gt, torch.bool, "crowd")
    _check(iou_sum, gt, torch.float64, "iou_sum")
    _require(pred.shape == gt.shape and gc.dim() == 2 and pc.dim() == 2 and gc.shape[0] == gt.shape[0]
             and pc.shape[0] == gt.shape[0] and crowd.shape == gc.shape, "incorrect input shapes")
    B, G, P = gt.shape[0], gc.shape[1], pc.shape[1]
    C = tp.shape[1] if reward else tp.numel()
    _require(0 < C < 2**31 - 1 and 0 < G < 2**31 - 1 and 0 < P < 2**31 - 1, "invalid capacities")
    _require(tuple(pairs.shape) == (B, G, P) and tuple(areas.shape) == (B, G + P) and matched.shape == gc.shape
             and error.numel() == 1, "incorrect scratch shapes")
    _require((tp.dim() == 2 and tp.shape[0] == B) if reward else tp.dim() == 1, "incorrect state shapes")
    _require(fp.shape == tp.shape and fn.shape == tp.shape and iou_sum.shape == tp.shape
             and (reward or tuple(confusion.shape) == (C, C + 1)), "incorrect state shapes")
    gt_ids, gt_slots = _lookup(gt_ids, gt_slots, gc, gt)
    pred_ids, pred_slots = _lookup(pred_ids, pred_slots, pc, gt)
    with torch.cuda.device(gt.device):
        return N.call("pe_update", N.ptr(gt), int(gt.dtype == torch.int64), N.ptr(pred),
                      int(pred.dtype == torch.int64), B, gt.shape[1] * gt.shape[2], N.ptr(gc), N.ptr(pc),
                      N.ptr(crowd), G, P, C, N.ptr(pairs), N.ptr(areas), N.ptr(matched), N.ptr(tp), N.ptr(fp),
                      N.ptr(fn), N.ptr(iou_sum), None if reward else N.ptr(confusion), N.ptr(gt_ids),
                      N.ptr(gt_slots), N.ptr(pred_ids), N.ptr(pred_slots), N.ptr(error), int(bool(validate)),
                      int(bool(reward)), N.stream_handle())


def _compute_rows(tp, fp, fn, sums, confusion, things, K, C):
    doubles = dict(dtype=torch.float64, device=tp.device)
    longs = dict(dtype=torch.int64, device=tp.device)
    values = torch.empty((K, 4, C), **doubles)
    summaries = torch.empty((K, 3, 3), **doubles)
    counts = torch.empty((K, 3), **longs)
    miou = torch.empty((K,), **doubles)
    copies = [torch.empty_like(t) for t in (tp, fp, fn, sums, confusion)]
    with torch.cuda.device(tp.device):
        N.call("pe_compute", N.ptr(tp), N.ptr(fp), N.ptr(fn), N.ptr(sums), N.ptr(confusion), N.ptr(things), K, C,
               N.ptr(values), N.ptr(summaries), N.ptr(counts), N.ptr(miou), *map(N.ptr, copies),
               N.stream_handle())
    return values, summaries, counts, miou, copies


def compute(tp, fp, fn, sums, confusion, things):
    """Summaries and independent snapshots (compute_kernel.cu:66-95)."""
    _require(tp.is_cuda and tp.dim() == 1 and 0 < tp.numel() < 2**31 - 1, "tp must be nonempty CUDA category counts")
    for t in (tp, fp, fn, sums, confusion, things):
        _require(t.device == tp.device and t.is_contiguous(), "incorrect device or layout")
    for t in (tp, fp, fn, confusion):
        _require(t.dtype == torch.int64, "counts must be int64")
    C = tp.numel()
    _require(fp.shape == tp.shape and fn.shape == tp.shape and sums.shape == tp.shape and things.shape == tp.shape
             and sums.dtype == torch.float64 and things.dtype == torch.bool
             and tuple(confusion.shape) == (C, C + 1), "incorrect state shapes or dtypes")
    values, summaries, counts, miou, copies = _compute_rows(tp, fp, fn, sums, confusion, things, 1, C)
    return [values[0], summaries[0], counts[0], miou[0], *copies]


def compute_prefix(tp, fp, fn, sums, confusion, things):
    """K independent rows (compute_kernel.cu:98-118)."""
    K, C = tp.shape
    values, summaries, counts, miou, copies = _compute_rows(tp, fp, fn, sums, confusion, things, K, C)
    return [values, summaries, counts, miou, *copies]


def pack(maps, ids, slots):
    """Original IDs -> compact slots (histogram_kernel.cu:343-366)."""
    _require(maps.is_cuda and maps.dim() == 3 and maps.is_contiguous() and maps.dtype in (torch.int32, torch.int64),
             "maps must be contiguous CUDA int32 or int64 B x H x W")
    _check(ids, maps, torch.int64, "lookup IDs")
    _check(slots, maps, torch.int32, "lookup slots")
    _require(ids.dim() == 2 and slots.shape == ids.shape and ids.shape[0] == maps.shape[0]
             and 0 < ids.shape[1] < 2**31 - 1, "incorrect lookup shapes")
    output = torch.empty(maps.shape, dtype=torch.int32, device=maps.device)
    error = torch.zeros(1, dtype=torch.int32, device=maps.device)
    with torch.cuda.device(maps.device):
        N.call("pe_pack", N.ptr(maps), int(maps.dtype == torch.int64), maps.shape[0], maps.shape[1] * maps.shape[2],
               N.ptr(ids), N.ptr(slots), ids.shape[1], N.ptr(output), N.ptr(error), N.stream_handle())
    return [output, error]
