"""Oracle: panoptic quality (PQ/SQ/RQ), semantic confusion/mIoU and per-image reward PQ.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``). A numpy restatement of
the reference CPU path in ``panoptic_evaluator/evaluator.py``.
"""

from __future__ import annotations

import numpy as np

INT64_MAX = np.iinfo(np.int64).max


def from_coco(maps, segments_info, category_ids):
    """Metadata tables for original segment IDs (evaluator.py:34-106).

    Returns ``(ids int64, slots int32, classes int32, crowd bool)``, each B x S
    with S = 1 + the largest segment count. Slot 0 is void; padding uses
    ``ids = INT64_MAX``, ``slots = 0``, ``classes = -1``.
    """
    maps = np.asarray(maps)
    if maps.ndim != 3 or maps.dtype not in (np.int32, np.int64):
        raise ValueError("maps must be integer B x H x W tensors")
    if len(segments_info) != maps.shape[0] or len(set(category_ids)) != len(category_ids):
        raise ValueError("batch length or category IDs are invalid")
    lookup = {category: index for index, category in enumerate(category_ids)}
    capacity = max((len(info) for info in segments_info), default=0) + 1
    ids_all, slots_all, classes_all, crowd_all = [], [], [], []
    for info in segments_info:
        ids = [entry["id"] for entry in info]
        if any(not isinstance(i, (int, np.integer)) or isinstance(i, bool) or i <= 0 or i >= INT64_MAX
               for i in ids) or len(set(ids)) != len(ids):
            raise ValueError("segment IDs must be unique positive int64 values below INT64_MAX; 0 is void")
        try:
            labels = [lookup[entry["category_id"]] for entry in info]
        except KeyError as error:
            raise ValueError("unknown category_id") from error
        padding = capacity - len(info) - 1
        ordered = sorted((int(identifier), slot) for slot, identifier in enumerate(ids, 1))
        ids_all.append([0] + [i for i, _ in ordered] + [INT64_MAX] * padding)
        slots_all.append([0] + [s for _, s in ordered] + [0] * padding)
        classes_all.append([-1] + labels + [-1] * padding)
        crowd_all.append([False] + [bool(entry.get("iscrowd", 0)) for entry in info] + [False] * padding)
    B = maps.shape[0]
    return (np.array(ids_all, dtype=np.int64).reshape(B, capacity),
            np.array(slots_all, dtype=np.int32).reshape(B, capacity),
            np.array(classes_all, dtype=np.int32).reshape(B, capacity),
            np.array(crowd_all, dtype=bool).reshape(B, capacity))


def decode_rgb(rgb):
    """COCO panoptic PNG pixels (B x H x W x 3 uint8) -> int64 IDs R + 256 G + 65536 B (README.md:68)."""
    rgb = np.asarray(rgb)
    if rgb.ndim != 4 or rgb.shape[-1] != 3 or rgb.dtype != np.uint8:
        raise ValueError("RGB maps must be uint8 B x H x W x 3")
    r, g, b = (rgb[..., k].astype(np.int64) for k in range(3))
    return r + 256 * g + 65536 * b


def encode_rgb(ids):
    """Inverse of decode_rgb for IDs below 2^24, as the reference tests write PNGs (test_evaluator.py:39)."""
    ids = np.asarray(ids, np.int64)
    return np.stack((ids % 256, ids // 256 % 256, ids // 65536 % 256), -1).astype(np.uint8)


def pack(maps, ids, slots):
    """Original IDs -> compact slots by binary search (evaluator.py:147-157)."""
    maps = np.asarray(maps)
    out = np.empty(maps.shape, dtype=np.int32)
    for b in range(maps.shape[0]):
        table = ids[b]
        image = maps[b].astype(np.int64)
        positions = np.minimum(np.searchsorted(table, image, side="left"), table.size - 1)
        found = slots[b][positions]
        valid = (table[positions] == image) & ((image == 0) | (found > 0))
        if not bool(valid.all()):
            raise ValueError("map contains a segment absent from segments_info")
        out[b] = found
    return out


def validate(maps, classes, crowd, num_classes, *, allow_empty_slots=False):
    """Host value checks of ``_prepare`` (evaluator.py:208-224)."""
    S = classes.shape[1]
    if maps.size and bool(((maps < 0) | (maps >= S)).any()):
        raise ValueError("segment map slot outside metadata capacity")
    if (bool(((classes < -1) | (classes >= num_classes)).any())
            or bool((classes[:, 0] != -1).any())
            or (crowd is not None and bool(crowd[:, 0].any()))):
        raise ValueError("classes must be -1 or valid category indices; slot 0 must be void")
    areas = slot_areas(maps, S)
    if allow_empty_slots:
        invalid = (areas[:, 1:] > 0) & (classes[:, 1:] < 0)
    else:
        invalid = (areas[:, 1:] > 0) != (classes[:, 1:] >= 0)
    if bool(invalid.any()):
        raise ValueError("nonvoid map slots and active metadata must correspond exactly")


def slot_areas(maps, S):
    """Per-image pixel count of every slot (evaluator.py:219-220)."""
    B = maps.shape[0]
    flat = maps.reshape(B, -1).astype(np.int64)
    offsets = np.arange(B, dtype=np.int64)[:, None] * S
    return np.bincount((flat + offsets).ravel(), minlength=B * S).reshape(B, S)


def histogram(gt, pred, G, P):
    """Pair histogram ``pairs[b, g, p]`` (evaluator.py:228-233)."""
    B = gt.shape[0]
    key = (np.arange(B, dtype=np.int64)[:, None, None] * G * P
           + gt.astype(np.int64) * P + pred.astype(np.int64))
    return np.bincount(key.ravel(), minlength=B * G * P).reshape(B, G, P).astype(np.int64)


def semantic(gt, pred, gc, pc, crowd, C):
    """Pixel confusion matrix C x (C+1); last column is predicted void (evaluator.py:236-243)."""
    B = gt.shape[0]
    g = gt.reshape(B, -1).astype(np.int64)
    p = pred.reshape(B, -1).astype(np.int64)
    target = np.take_along_axis(gc.astype(np.int64), g, 1)
    prediction = np.take_along_axis(pc.astype(np.int64), p, 1)
    valid = (target >= 0) & ~np.take_along_axis(crowd, g, 1)
    prediction = np.where(prediction >= 0, prediction, C)
    keys = (target * (C + 1) + prediction)[valid]
    return np.bincount(keys, minlength=C * (C + 1)).reshape(C, C + 1).astype(np.int64)


def match_statistics(pairs, gc, pc, crowd, *, reward=False):
    """Per-segment PQ decisions from a pair histogram (evaluator.py:383-404, 522-534).

    Returns ``(pm [B,P] bool, fp [B,P] bool, fn [B,G] bool, iou_per_pred [B,P] f64, ga, pa)``.
    """
    ga = pairs.sum(2)
    pa = pairs.sum(1)
    union = ga[:, :, None] + pa[:, None, :] - pairs - pairs[:, :1, :]
    iou = pairs.astype(np.float64) / np.maximum(union, 1)
    same = (gc[:, :, None] == pc[:, None, :]) & (gc[:, :, None] >= 0)
    matches = same & ~crowd[:, :, None] & (iou > 0.5)
    gm, pm = matches.any(2), matches.any(1)
    G = gc.shape[1]
    slots = np.arange(G)[None, :, None]
    same_crowd = crowd[:, :, None] & same
    last = np.where(same_crowd, slots, -1).max(1) if G else np.full(pc.shape, -1)
    overlap = np.take_along_axis(pairs, np.maximum(last, 0)[:, None, :], 1)[:, 0, :]
    ignored_area = pairs[:, 0, :] + np.where(last >= 0, overlap, 0)
    false_positive = (pc >= 0) & ~pm & (ignored_area.astype(np.float64) <= 0.5 * pa)
    if reward:
        false_positive &= pa > 0
    false_negative = (gc >= 0) & ~crowd & ~gm
    iou_per_pred = (iou * matches).sum(1)
    return pm, false_positive, false_negative, iou_per_pred, ga, pa


class PanopticOracle:
    """Dataset accumulator mirroring ``PanopticEvaluator`` on CPU (evaluator.py:246-468)."""

    def __init__(self, num_classes, isthing=None, validate=True):
        self.num_classes = num_classes
        self.isthing = np.array(isthing if isthing is not None else [True] * num_classes, dtype=bool)
        self.validate = validate
        self.reset()

    def reset(self):
        C = self.num_classes
        self.tp = np.zeros(C, np.int64)
        self.fp = np.zeros(C, np.int64)
        self.fn = np.zeros(C, np.int64)
        self.iou_sum = np.zeros(C, np.float64)
        self.confusion = np.zeros((C, C + 1), np.int64)

    def update(self, pred, pc, gt, gc, crowd=None, *, return_areas=False):
        """Compact-slot update (evaluator.py:291-379 CPU branch, :381-417)."""
        gt, pred = np.asarray(gt), np.asarray(pred)
        gc, pc = np.asarray(gc, np.int32), np.asarray(pc, np.int32)
        crowd = np.zeros(gc.shape, bool) if crowd is None else np.asarray(crowd, bool)
        if self.validate:
            validate(gt, gc, crowd, self.num_classes)
            validate(pred, pc, None, self.num_classes)
        if gt.shape != pred.shape:
            raise ValueError("prediction and target must share shape and evaluator device")
        C = self.num_classes
        pairs = histogram(gt, pred, gc.shape[1], pc.shape[1])
        conf = semantic(gt, pred, gc, pc, crowd, C)
        pm, fp, fn, iou_pp, ga, _ = match_statistics(pairs, gc, pc, crowd)
        np.add.at(self.tp, np.maximum(pc, 0).ravel(), pm.ravel().astype(np.int64))
        np.add.at(self.fp, np.maximum(pc, 0).ravel(), fp.ravel().astype(np.int64))
        np.add.at(self.fn, np.maximum(gc, 0).ravel(), fn.ravel().astype(np.int64))
        np.add.at(self.iou_sum, np.maximum(pc, 0).ravel(), iou_pp.ravel())
        self.confusion += conf
        return ga if return_areas else self

    def compute(self):
        return compute(self.tp, self.fp, self.fn, self.iou_sum, self.confusion, self.isthing)


def compute(tp, fp, fn, iou_sum, confusion, isthing):
    """PQ/SQ/RQ, group means and semantic IoU (evaluator.py:448-468)."""
    C = tp.shape[0]
    denom = tp.astype(np.float64) + 0.5 * (fp + fn).astype(np.float64)
    pq = iou_sum / np.maximum(denom, 1)
    sq = iou_sum / np.maximum(tp, 1)
    rq = tp / np.maximum(denom, 1)
    active = denom > 0

    def average(mask):
        selected = mask & active
        n = selected.sum()
        d = max(int(n), 1)
        return {"pq": (pq * selected).sum() / d, "sq": (sq * selected).sum() / d,
                "rq": (rq * selected).sum() / d, "n": np.int64(n)}

    diagonal = np.diagonal(confusion[:, :C]).copy()
    union = confusion.sum(1) + confusion[:, :C].sum(0) - diagonal
    with np.errstate(invalid="ignore", divide="ignore"):
        semantic_iou = np.where(union > 0, diagonal.astype(np.float64) / np.maximum(union, 1), np.nan)
    miou = np.nan_to_num(semantic_iou, nan=0.0).sum() / max(int((union > 0).sum()), 1)
    return {"All": average(np.ones(C, bool)), "Things": average(isthing), "Stuff": average(~isthing),
            "per_class": {"pq": pq, "sq": sq, "rq": rq, "iou": semantic_iou},
            "miou": np.float64(miou), "tp": tp.copy(), "fp": fp.copy(), "fn": fn.copy(),
            "iou_sum": iou_sum.copy(), "confusion": confusion.copy()}


def reward_statistics(pred, pc, gt, gc, crowd, num_classes, *, validate_inputs=True):
    """Per-image [B, C] (iou_sum, tp, fp, fn) for ``panoptic_quality`` (evaluator.py:484-538)."""
    gt, pred = np.asarray(gt), np.asarray(pred)
    gc, pc = np.asarray(gc, np.int32), np.asarray(pc, np.int32)
    crowd = np.zeros(gc.shape, bool) if crowd is None else np.asarray(crowd, bool)
    if validate_inputs:
        validate(gt, gc, crowd, num_classes)
        validate(pred, pc, None, num_classes, allow_empty_slots=True)
    if gt.shape != pred.shape:
        raise ValueError("prediction and target must share shape and device")
    B, C = gt.shape[0], num_classes
    pairs = histogram(gt, pred, gc.shape[1], pc.shape[1])
    pm, fp, fn, iou_pp, _, _ = match_statistics(pairs, gc, pc, crowd, reward=True)
    tp_o = np.zeros((B, C), np.int64)
    fp_o = np.zeros((B, C), np.int64)
    fn_o = np.zeros((B, C), np.int64)
    sums = np.zeros((B, C), np.float64)
    for b in range(B):
        np.add.at(tp_o[b], np.maximum(pc[b], 0), pm[b].astype(np.int64))
        np.add.at(fp_o[b], np.maximum(pc[b], 0), fp[b].astype(np.int64))
        np.add.at(fn_o[b], np.maximum(gc[b], 0), fn[b].astype(np.int64))
        np.add.at(sums[b], np.maximum(pc[b], 0), iou_pp[b])
    return sums, tp_o, fp_o, fn_o


def panoptic_quality(pred, pc, gt, gc, crowd, num_classes, *, validate_inputs=True, return_stats=False):
    """Mean-class PQ per image (evaluator.py:471-544)."""
    sums, tp, fp, fn = reward_statistics(pred, pc, gt, gc, crowd, num_classes,
                                         validate_inputs=validate_inputs)
    if return_stats:
        return np.stack((sums, tp.astype(np.float64), fp.astype(np.float64), fn.astype(np.float64)), -1)
    denominator = tp.astype(np.float64) + 0.5 * (fp + fn).astype(np.float64)
    active = denominator > 0
    pq = sums / np.maximum(denominator, 1)
    return pq.sum(1) / np.maximum(active.sum(1), 1)
