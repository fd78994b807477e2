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
    if R:
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
    descs = table[T8: T8 + D8].view(torch.int64)
    step_q = table[T8 + D8: T8 + D8 + 4 * steps.size].view(torch.int32)
    # Every output is a view of one 8-byte-element allocation (the last element: the owner pass's
    # chunk counter, zeroed by the call), every int32 workspace of another.
    shapes = (("tp", (R, C), torch.int64), ("fp", (R, C), torch.int64), ("fn", (R, C), torch.int64),
              ("sums", (R, C), torch.float64), ("confusion", (R, C, C + 1), torch.int64),
              ("itp", (R, T, C), torch.int64), ("ifp", (R, T, C), torch.int64), ("ifn", (R, T, C), torch.int64),
              ("precision", (R, T, C), torch.float64), ("recall", (R, T, C), torch.float64),
              ("values", (R, 4, C), torch.float64), ("summaries", (R, 3, 3), torch.float64),
              ("counts", (R, 3), torch.int64), ("miou", (R,), torch.float64))
    sizes = [math.prod(shape) for _, shape, _ in shapes]
    parts = torch.empty(sum(sizes) + 1, dtype=torch.int64, device=dev).split(sizes + [1])
    out = {key: (part if dtype is torch.int64 else part.view(dtype)).view(shape)
           for (key, shape, dtype), part in zip(shapes, parts)}
    schedule = parts[-1]
    classes_flat = (torch.cat([c.reshape(-1) for c in classes]).to(torch.int32) if n.sum()
                    else torch.empty(0, dtype=torch.int32, device=dev))
    work = [B * S, max(int((n * S).sum()), 1), max(int(cells.sum()), 1), B * T * C * 2, 1]
    ints = torch.empty(sum(work), dtype=torch.int32, device=dev)
    ga, raw, pairs, counters, error = ints.split(work)  # error is zeroed by the call
    things = isthing.to(torch.uint8)
    crowd_u8 = crowd.reshape(-1).view(torch.uint8)
    with N.on_device(dev):
        code = N.call("pe_prefix", N.ptr(descs), B, int(chunks * B), R, S, int(n.max()) + 1,
                      int((S * (n + 1)).max()), N.ptr(step_q), N.ptr(classes_flat),
                      N.ptr(gc.reshape(-1)), N.ptr(crowd_u8), N.ptr(things), N.ptr(thr), T, C, N.ptr(ga), ga.numel(),
                      N.ptr(raw), int((n * S).sum()), N.ptr(pairs), int(cells.sum()), N.ptr(counters),
                      counters.numel(), N.ptr(out["tp"]), N.ptr(out["fp"]), N.ptr(out["fn"]), N.ptr(out["sums"]),
                      N.ptr(out["confusion"]), N.ptr(out["itp"]), N.ptr(out["ifp"]), N.ptr(out["ifn"]),
                      N.ptr(out["precision"]), N.ptr(out["recall"]), N.ptr(out["values"]), N.ptr(out["summaries"]),
                      N.ptr(out["counts"]), N.ptr(out["miou"]), int(bool(validate)),
                      int(BULK_PASS), N.ptr(schedule) if BULK_PASS else None, N.ptr(error),
                      N.stream_handle(dev))
    # Keep inputs referenced by raw pointers alive until the work is queued.
    del masks
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
