"""Oracle: generation-order prefix evaluation (canvas PQ/mIoU + greedy instance P/R).

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``). Restates the CPU
branch of ``panoptic_evaluator/prefix.py`` (prefix.py:12-122).
"""

from __future__ import annotations

import math

import numpy as np

from . import panoptic as pan


def check_arguments(thresholds, checkpoints):
    """Argument checks (prefix.py:31-39)."""
    thresholds = tuple(thresholds)
    if not thresholds or any(isinstance(t, bool) or not math.isfinite(t) or not 0 < t <= 1
                             for t in thresholds):
        raise ValueError("iou_thresholds must be finite values in (0, 1]")
    requested = None if checkpoints is None else tuple(checkpoints)
    if requested is not None and (any(type(k) is not int or k < 0 for k in requested)
                                  or any(a >= b for a, b in zip(requested, requested[1:]))):
        raise ValueError("checkpoints must be strictly increasing nonnegative integers")
    return np.array(thresholds, np.float64), requested


def image_prefixes(gt, gc, crowd, masks, classes, isthing, num_classes, thresholds, points):
    """Snapshots for one image (prefix.py:63-120).

    ``gt`` is an H x W compact slot map, ``masks`` N x H x W bool in generation order.
    Returns a list of dicts with the fields of ``segmentation_prefixes``.
    """
    C = num_classes
    n, g = len(masks), gc.shape[0]
    labels = np.concatenate(([-1], np.asarray(classes, np.int64)))
    canvas = np.zeros(gt.shape, np.int64)
    gtl = gt.astype(np.int64)
    ga = np.bincount(gtl.ravel(), minlength=g)
    pairs = np.zeros((g, n + 1), np.int64)
    pairs[:, 0] = ga
    T = len(thresholds)
    tp = np.zeros((T, C), np.int64)
    fp = np.zeros((T, C), np.int64)
    used = np.zeros((T, g), bool)
    things = (gc >= 0) & isthing[np.maximum(gc, 0)]
    positives = np.zeros(C, np.int64)
    np.add.at(positives, np.maximum(gc, 0), (things & ~crowd).astype(np.int64))
    pixel_areas = masks.reshape(n, gt.size).sum(1).astype(np.float64)
    snapshots = []

    def snapshot(k):
        valid = (gc >= 0) & ~crowd
        active = np.where(pairs.sum(0) > 0, labels, -1)
        columns = np.where(active >= 0, active, C)
        confusion = np.zeros((C, C + 1), np.int64)
        idx = gc[valid][:, None].astype(np.int64) * (C + 1) + columns[None]
        np.add.at(confusion.reshape(-1), idx.ravel(), pairs[valid].ravel())
        pm, fpm, fnm, iou_pp, _, _ = pan.match_statistics(pairs[None], gc[None], active[None].astype(np.int64),
                                                          crowd[None])
        e_tp = np.zeros(C, np.int64)
        e_fp = np.zeros(C, np.int64)
        e_fn = np.zeros(C, np.int64)
        e_sum = np.zeros(C, np.float64)
        np.add.at(e_tp, np.maximum(active, 0), pm[0].astype(np.int64))
        np.add.at(e_fp, np.maximum(active, 0), fpm[0].astype(np.int64))
        np.add.at(e_fn, np.maximum(gc, 0), fnm[0].astype(np.int64))
        np.add.at(e_sum, np.maximum(active, 0), iou_pp[0])
        result = pan.compute(e_tp, e_fp, e_fn, e_sum, confusion, isthing)
        result["prefix"] = k
        result["instance"] = dict(
            iou_thresholds=thresholds.copy(), tp=tp.copy(), fp=fp.copy(), fn=positives[None] - tp,
            precision=tp.astype(np.float64) / np.maximum(tp + fp, 1),
            recall=tp.astype(np.float64) / np.maximum(positives, 1)[None])
        snapshots.append(result)

    if 0 in points:
        snapshot(0)
    for i in range(n):
        mask = masks[i]
        covered, previous = gtl[mask], canvas[mask]
        inter = np.bincount(covered, minlength=g)
        np.add.at(pairs.reshape(-1), covered * (n + 1) + previous, -1)
        pairs[:, i + 1] = inter
        canvas[mask] = i + 1
        c = int(classes[i])
        if bool(isthing[c]):
            area = pixel_areas[i]
            union = np.where(crowd, area, area + ga - inter)
            ious = inter.astype(np.float64) / np.maximum(union, 1)
            same = gc == c
            eligible = same[None] & ~crowd[None] & ~used & (ious[None] >= thresholds[:, None])
            scored = np.where(eligible, ious[None], -1.0)
            best = scored.argmax(1)  # first maximum, as torch.max on CPU
            best_iou = scored[np.arange(T), best]
            matched = best_iou >= 0
            used[np.arange(T), best] |= matched
            ignored = (same[None] & crowd[None] & (ious[None] >= thresholds[:, None])).any(1)
            tp[:, c] += matched.astype(np.int64)
            fp[:, c] += (~matched & ~ignored).astype(np.int64)
        if i + 1 in points:
            snapshot(i + 1)
    return snapshots


def segmentation_prefixes(masks_list, classes_list, gt, gc, crowd, num_classes, *, isthing=None,
                          checkpoints=None, iou_thresholds=(0.5, 0.75), validate=True):
    """Batch driver (prefix.py:12-122) on compact targets."""
    thresholds, requested = check_arguments(iou_thresholds, checkpoints)
    gt = np.asarray(gt)
    gc = np.asarray(gc, np.int32)
    crowd = np.zeros(gc.shape, bool) if crowd is None else np.asarray(crowd, bool)
    isthing = np.array(isthing if isthing is not None else [True] * num_classes, bool)
    if validate:
        pan.validate(gt, gc, crowd, num_classes)
        for b in range(len(masks_list)):
            cl = np.asarray(classes_list[b])
            if ((cl < 0) | (cl >= num_classes)).any():
                raise ValueError("classes must be valid category indices")
            m = np.asarray(masks_list[b], bool)
            if len(m) and (m.reshape(len(m), -1).sum(1) == 0).any():
                raise ValueError("each instance mask must have pixels")
    if len(masks_list) != len(gt) or any(np.asarray(m).shape[1:] != gt.shape[1:] for m in masks_list):
        raise ValueError("prediction and target must have matching batch and image dimensions")
    if requested and any(requested[-1] > len(m) for m in masks_list):
        raise ValueError("checkpoint exceeds prediction count")
    results = []
    for b in range(len(masks_list)):
        masks = np.asarray(masks_list[b], bool)
        n = len(masks)
        points = set(requested if requested is not None else (range(1, n + 1) if n else [0]))
        results.append(image_prefixes(gt[b], gc[b], crowd[b], masks, np.asarray(classes_list[b]),
                                      isthing, num_classes, thresholds, points))
    return results
