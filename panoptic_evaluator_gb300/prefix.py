"""Generation-order prefix evaluation on the GPU (API of the reference's ``prefix.py``).

``segmentation_prefixes`` evaluates every image of the batch with one
``pe_prefix`` call (six launches in total): a single pass over each image's
target map and mask bytes, a scan, per-checkpoint canvas scoring, per-image
greedy matching and the per-checkpoint summaries. Results are views of
device tensors, one list of snapshots per image; a snapshot makes the views of
its fields when they are read.
"""

from __future__ import annotations

import itertools
import math
from collections.abc import Mapping

import numpy as np
import torch

from . import _native as N
from ._batch import check_pixels
from .evaluator import PanopticBatch, _prepare
from .instance import InstanceBatch, check_instance_batch, shape_table

FIELDS = 16
(TARGET, MASKS, PIXELS, STRIDE, CHUNK_BEGIN, NMASK, NSLOT, DET_BEGIN, SLOT_BEGIN, Q_BEGIN, NQ, PAIR_BEGIN, RAW_BEGIN,
 FLAGS, STEP_BEGIN, COUNT_BEGIN) = range(FIELDS)
CHUNK = 4096

# The owner pass streams mask segments through a bulk-copy ring (rows at any
# alignment); set False to use the register-load pass instead.
BULK_PASS = True

_ERRORS = (
    (1 | 2, "unknown target slot or empty prediction mask"),
    (4, "classes must be -1 or valid category indices; slot 0 must be void"),
    (8, "nonvoid map slots and active metadata must correspond exactly"),
    (16, "classes must be valid category indices"),
)


def _check_arguments(iou_thresholds, checkpoints):
    """Argument checks of the reference (prefix.py:31-39)."""
    thresholds = tuple(iou_thresholds)
    if not thresholds or any(isinstance(t, bool) or not math.isfinite(t) or not 0 < t <= 1 for t in thresholds):
        raise ValueError("iou_thresholds must be finite values in (0, 1]")
    requested = None if checkpoints is None else tuple(checkpoints)
    if requested is not None and (any(type(k) is not int or k < 0 for k in requested)
                                  or any(a >= b for a, b in zip(requested, requested[1:]))):
        raise ValueError("checkpoints must be strictly increasing nonnegative integers")
    return thresholds, requested


_CONSTANTS: dict = {}


def _device_constant(values, dtype, device):
    """Small per-call constants (thresholds, thing flags) uploaded once per device and reused."""
    key = (tuple(values), dtype, str(device))
    tensor = _CONSTANTS.get(key)
    if tensor is None:
        if len(_CONSTANTS) > 256:
            _CONSTANTS.clear()
        tensor = _CONSTANTS[key] = torch.tensor(values, dtype=dtype, device=device)
    return tensor


def _aligned(ptr, stride=0):
    return ptr % 16 == 0 and stride % 16 == 0


_OUTPUT_FIELDS = (("tp", 1, torch.int64), ("fp", 1, torch.int64), ("fn", 1, torch.int64), ("sums", 1, torch.float64),
                  ("confusion", 2, torch.int64), ("itp", 3, torch.int64), ("ifp", 3, torch.int64),
                  ("ifn", 3, torch.int64), ("precision", 3, torch.float64), ("recall", 3, torch.float64),
                  ("values", 4, torch.float64), ("summaries", 5, torch.float64), ("counts", 6, torch.int64),
                  ("miou", 7, torch.float64))
_LAYOUTS: dict = {}


def _output_layout(R, T, C):
    """key -> (offset in 8-byte elements, shape, dtype) of pe_prefix's outputs for R rows, and the total size."""
    key = (R, T, C)
    cached = _LAYOUTS.get(key)
    if cached is None:
        shapes = {1: (R, C), 2: (R, C, C + 1), 3: (R, T, C), 4: (R, 4, C), 5: (R, 3, 3), 6: (R, 3), 7: (R,)}
        layout, offset = {}, 0
        for name, kind, dtype in _OUTPUT_FIELDS:
            layout[name] = (offset, shapes[kind], dtype)
            offset += math.prod(shapes[kind])
        cached = _LAYOUTS[key] = (layout, offset)
        if len(_LAYOUTS) > 256:
            _LAYOUTS.pop(next(iter(_LAYOUTS)))
    return cached


class PackedOutputs(Mapping):
    """pe_prefix's outputs: named views of one int64 allocation, each made on first access and kept."""

    __slots__ = ("flat", "_layout", "_views")

    def __init__(self, flat, layout):
        self.flat, self._layout, self._views = flat, layout, {}

    def __getitem__(self, key):
        view = self._views.get(key)
        if view is None:
            offset, shape, dtype = self._layout[key]
            part = self.flat[offset: offset + math.prod(shape)]
            view = self._views[key] = (part if dtype is torch.int64 else part.view(dtype)).view(shape)
        return view

    def __iter__(self):
        return iter(self._layout)

    def __len__(self):
        return len(self._layout)


def run_prefixes(maps, gc, crowd, masks, classes, num_classes, isthing, thresholds, points, validate,
                 masks_per_image=None):
    """Launch pe_prefix for B images. masks/classes: per-image lists; points: per-image checkpoint lists.

    Returns the output tensors (rows = all checkpoints of all images in order) and the row offsets.
    masks_per_image: the mask counts as an int64 array, when the caller has them.
    """
    dev = maps.device
    B, H, W = maps.shape
    HW = H * W
    S = gc.shape[1]
    T, C = len(thresholds), num_classes
    n = np.fromiter((m.shape[0] for m in masks), np.int64, B) if masks_per_image is None else masks_per_image
    q = np.fromiter(map(len, points), np.int64, B)
    d = np.zeros((B, FIELDS), np.int64)
    img = np.arange(B, dtype=np.int64)
    d[:, TARGET] = maps.data_ptr() + img * HW * 4
    d[:, MASKS] = [m.data_ptr() for m in masks]
    check_pixels(HW)
    d[:, PIXELS] = HW
    d[:, STRIDE] = HW
    chunks = -(-HW // CHUNK)
    d[:, CHUNK_BEGIN] = img * chunks
    d[:, NMASK] = n
    d[:, NSLOT] = S
    d[:, DET_BEGIN] = np.cumsum(n) - n
    d[:, SLOT_BEGIN] = img * S
    d[:, Q_BEGIN] = np.cumsum(q) - q
    d[:, NQ] = q
    cells = q * S * (n + 1)
    d[:, PAIR_BEGIN] = np.cumsum(cells) - cells
    d[:, RAW_BEGIN] = np.cumsum(n * S) - n * S
    maps_vec = _aligned(maps.data_ptr()) and HW % 4 == 0
    d[:, FLAGS] = [int(maps_vec) | 2 * int(_aligned(m.data_ptr(), HW)) for m in masks]
    d[:, STEP_BEGIN] = np.cumsum(n + 1) - (n + 1)
    d[:, COUNT_BEGIN] = img * T * C * 2
    # steps[STEP_BEGIN[b] + k] = index of checkpoint k among image b's checkpoints, -1 elsewhere.
    steps = np.full(int((n + 1).sum()), -1, np.int32)
    R = int(q.sum())
    if R and all(p == points[0] for p in points):  # the same checkpoints for every image (one broadcast)
        first = np.asarray(points[0], np.int64)
        steps[(d[:, STEP_BEGIN, None] + first).ravel()] = np.tile(np.arange(first.size, dtype=np.int32), B)
    elif R:
        flat_points = np.fromiter(itertools.chain.from_iterable(points), np.int64, R)
        first_row = np.cumsum(q) - q
        steps[np.repeat(d[:, STEP_BEGIN], q) + flat_points] = np.arange(R) - np.repeat(first_row, q)
    # One pinned upload: thresholds (f64), descriptors (int64), then the step table (int32).
    T8, D8 = 8 * T, 8 * B * FIELDS
    host = torch.empty(T8 + D8 + 4 * steps.size + 8, dtype=torch.uint8, pin_memory=True)
    view = host.numpy()
    view[:T8] = np.asarray(thresholds, np.float64).view(np.uint8)
    view[T8: T8 + D8] = d.reshape(-1).view(np.uint8)
    view[T8 + D8: T8 + D8 + 4 * steps.size] = steps.view(np.uint8)
    table = host.to(dev, non_blocking=True)
    thr = table[:T8].view(torch.float64)  # fresh per call: results never alias a cache
    table_ptr = table.data_ptr()  # thresholds, then descriptors (int64), then the step table (int32)
    # Every output is a view of one 8-byte-element allocation (the last element: the owner pass's
    # chunk counter, zeroed by the call), made when first read; the kernels get pointers into it.
    layout, total = _output_layout(R, T, C)
    flat = torch.empty(total + 1, dtype=torch.int64, device=dev)
    out = PackedOutputs(flat, layout)
    base = flat.data_ptr()
    at = {key: base + 8 * offset for key, (offset, _, _) in layout.items()}
    total_masks, max_masks = int(n.sum()), int(n.max())
    classes_flat = (torch.cat(classes).to(torch.int32) if total_masks
                    else torch.empty(0, dtype=torch.int32, device=dev))
    raw_len, pairs_len = S * total_masks, int(cells.sum())
    # int32 workspaces, one allocation: ga [B x S], raw, pairs, counters [B x T x C x 2], error (zeroed by the call).
    work = (B * S, max(raw_len, 1), max(pairs_len, 1), B * T * C * 2, 1)
    workspace = torch.empty(sum(work), dtype=torch.int32, device=dev)  # referenced until the call is queued
    ints = workspace.data_ptr()
    ga, raw, pairs, counters, error = (ints + 4 * sum(work[:i]) for i in range(5))
    things = isthing.to(torch.uint8)
    with N.on_device(dev):
        code = N.call("pe_prefix", table_ptr + T8, B, int(chunks * B), R, S, max_masks + 1, S * (max_masks + 1),
                      table_ptr + T8 + D8, N.ptr(classes_flat), N.ptr(gc), N.ptr(crowd), N.ptr(things), table_ptr,
                      T, C, ga, work[0], raw, raw_len, pairs, pairs_len, counters, work[3], at["tp"], at["fp"],
                      at["fn"], at["sums"], at["confusion"], at["itp"], at["ifp"], at["ifn"], at["precision"],
                      at["recall"], at["values"], at["summaries"], at["counts"], at["miou"], int(bool(validate)),
                      int(BULK_PASS), base + 8 * total if BULK_PASS else None, error, N.stream_handle(dev))
    # Keep inputs and workspaces referenced by raw pointers alive until the work is queued.
    del masks, workspace, classes_flat
    return out, d[:, Q_BEGIN], int(code) if validate else 0, thr


def raise_prefix_error(code):
    for bits, message in _ERRORS:
        if code & bits:
            raise ValueError(message)


_GROUPS = ("All", "Things", "Stuff")
_METRICS = ("pq", "sq", "rq", "iou")
_ROW_FIELDS = {"tp": "tp", "fp": "fp", "fn": "fn", "iou_sum": "sums", "confusion": "confusion", "miou": "miou"}


class Snapshot(Mapping):
    """One checkpoint's result dict (prefix.py:125-142), built lazily from the call's packed outputs.

    Keys: ``prefix``, ``All`` / ``Things`` / ``Stuff`` ({pq, sq, rq, n}),
    ``miou``, ``tp``, ``fp``, ``fn``, ``iou_sum``, ``confusion``,
    ``per_class`` ({pq, sq, rq, iou}) and ``instance`` ({iou_thresholds, tp,
    fp, fn, precision, recall}). Every value is a view of row ``row`` of the
    packed output tensors, made when the key is first read and kept, so a
    caller that reads a few keys of a few checkpoints creates a few views and
    not every field of every row.
    """

    __slots__ = ("_out", "_row", "_prefix", "_thr", "_cache")
    _KEYS = ("All", "Things", "Stuff", "prefix", "miou", "tp", "fp", "fn", "iou_sum", "confusion", "per_class",
             "instance")

    def __init__(self, out, row, prefix, thr):
        self._out, self._row, self._prefix, self._thr = out, row, prefix, thr
        self._cache = {}

    def __getitem__(self, key):
        cache = self._cache
        if key in cache:
            return cache[key]
        out, r = self._out, self._row
        if key == "prefix":
            value = self._prefix
        elif key in _ROW_FIELDS:
            value = out[_ROW_FIELDS[key]][r]
        elif key in _GROUPS:
            i = _GROUPS.index(key)
            summary, counts = out["summaries"][r, i], out["counts"][r]
            value = dict(pq=summary[0], sq=summary[1], rq=summary[2], n=counts[i])
        elif key == "per_class":
            value = dict(zip(_METRICS, out["values"][r].unbind(0)))
        elif key == "instance":
            value = dict(iou_thresholds=self._thr, tp=out["itp"][r], fp=out["ifp"][r], fn=out["ifn"][r],
                         precision=out["precision"][r], recall=out["recall"][r])
        else:
            raise KeyError(key)
        cache[key] = value
        return value

    def __iter__(self):
        return iter(self._KEYS)

    def __len__(self):
        return len(self._KEYS)

    def __repr__(self):
        return f"Snapshot(prefix={self._prefix}, row={self._row})"


def unpack(out, row, points, thr):
    """One lazy result dict per checkpoint of one image, rows row, row + 1, ..."""
    return [Snapshot(out, row + offset, k, thr) for offset, k in enumerate(points)]


def check_prefix_inputs(masks, classes, maps_shape, device, requested):
    """Structural checks of the predictions (prefix.py:41-48): the instance checks of each image's masks and
    classes (with their messages, instance.py:78-126), then the batch size and image dimensions against the
    B x H x W target maps and the checkpoints (`requested`, or None) against the mask counts.

    Returns the per-image mask counts (int64 array), or None for an empty batch.
    """
    shapes, _ = check_instance_batch(InstanceBatch(masks, classes), device, prediction=False)
    if len(masks) != maps_shape[0]:
        raise ValueError("prediction and target must have matching batch and image dimensions")
    if not masks:
        return None
    table = shape_table(shapes)
    if (table[:, 1] != maps_shape[1]).any() or (table[:, 2] != maps_shape[2]).any():
        raise ValueError("prediction and target must have matching batch and image dimensions")
    counts = table[:, 0]
    if requested and requested[-1] > int(counts.min()):
        raise ValueError("checkpoint exceeds prediction count")
    return counts


@torch.no_grad()
def segmentation_prefixes(prediction: InstanceBatch, target: PanopticBatch, num_classes, *, isthing=None,
                          checkpoints=None, iou_thresholds=(0.5, 0.75), validate=True):
    """Evaluate independent masks in generation order, later masks drawn on top (prefix.py:12-27).

    Returns one list per image of snapshot dicts with ``prefix``, the
    panoptic/semantic results of the canvas and ``instance`` counts /
    precision / recall of shape [threshold, class].
    """
    if not isinstance(num_classes, int) or isinstance(num_classes, bool) or num_classes <= 0:
        raise ValueError("num_classes must be a positive integer")
    thresholds, requested = _check_arguments(iou_thresholds, checkpoints)
    device = target.segment_map.device
    if device.type != "cuda":
        raise ValueError("pe_gb300 evaluates on CUDA devices only")
    things = _device_constant(tuple(bool(x) for x in isthing) if isthing is not None else (True,) * num_classes,
                              torch.uint8, device)
    if len(things) != num_classes:
        raise ValueError("isthing must contain one flag per category")
    target = target.compact()
    if target.crowd is None:
        from dataclasses import replace
        target = replace(target, crowd=torch.zeros_like(target.classes, dtype=torch.bool))
    maps, gc, crowd = _prepare(target, num_classes)
    masks = list(prediction.masks)
    classes = list(prediction.classes)
    counts = check_prefix_inputs(masks, classes, tuple(maps.shape), device, requested)
    if counts is None:
        return []
    points = [list(requested) if requested is not None else (list(range(1, len(m) + 1)) if len(m) else [0])
              for m in masks]
    masks = [m.contiguous() for m in masks]
    out, rows, code, thr = run_prefixes(maps, gc, crowd, masks, classes, num_classes, things, thresholds, points,
                                        validate, counts)
    if validate:
        raise_prefix_error(code)
    return [unpack(out, int(rows[b]), points[b], thr) for b in range(len(masks))]
