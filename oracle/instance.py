"""Oracle: COCO mask AP/AR (greedy matching and 101-point precision/recall).

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``). A numpy / plain-Python
restatement of ``panoptic_evaluator/instance.py``. The matcher is a literal
triple loop and is meant for small cases.
"""

from __future__ import annotations

import numpy as np

# instance.py:251-252
RANGES = ((0.0, 1e10), (0.0, 1024.0), (1024.0, 9216.0), (9216.0, 1e10))
IOU_THRESHOLDS = (0.5, 0.55, 0.6, 0.65, 0.7, 0.75, 0.8, 0.85, 0.8999999999999999, 0.95)
MAX_DETECTIONS = (1, 10, 100)


def score_order(scores):
    """Stable descending argsort (instance.py:140, :213)."""
    return np.argsort(-np.asarray(scores, np.float64), kind="stable")


def mask_ious(pm, gm, pa, ga, crowd):
    """Pairwise mask IoU; crowd targets use the detection area (instance.py:255-264)."""
    d, g = len(pm), len(gm)
    inter = np.zeros((d, g), np.float64)
    if d and g:
        p = pm.reshape(d, -1).astype(np.float32)
        q = gm.reshape(g, -1).astype(np.float32)
        assert p.shape[1] < 2**24, "float32 products are exact only below 2**24 pixels"
        inter = (p @ q.T).astype(np.float64)  # exact: counts < 2**24
    union = np.where(crowd[None], pa[:, None], pa[:, None] + ga[None] - inter)
    return inter / np.maximum(union, 1)


def match_ious(ious, pc, gc, pa, crowd, areas, classes):
    """COCO greedy matching for 4 area ranges x 10 thresholds (instance.py:267-297).

    ``pc``, ``pa`` are score-sorted detections. Returns ``(status int8 [40, D],
    ranks int32 [D], counts int64 [classes, 4])``.
    """
    pc = np.asarray(pc)
    gc = np.asarray(gc)
    crowd = np.asarray(crowd, bool)
    areas = np.asarray(areas, np.float64)
    pa = np.asarray(pa, np.float64)
    d = len(pc)
    status = np.full((40, d), -1, np.int8)
    ranks = np.zeros(d, np.int32)
    counts = np.zeros((classes, 4), np.int64)
    for c in range(classes):
        ds = np.nonzero(pc == c)[0].tolist()[:100]
        for rank, i in enumerate(ds):
            ranks[i] = rank + 1
        gs = np.nonzero(gc == c)[0].tolist()
        for a, (low, high) in enumerate(RANGES):
            ignored = crowd | (areas < low) | (areas > high)
            ordered = sorted(gs, key=lambda j: bool(ignored[j]))
            counts[c, a] = sum(not bool(ignored[j]) for j in gs)
            for t in range(10):
                used = set()
                for i in ds:
                    best, overlap = -1, IOU_THRESHOLDS[t]
                    for j in ordered:
                        if j in used and not crowd[j]:
                            continue
                        if best >= 0 and not ignored[best] and ignored[j]:
                            break
                        if ious[i, j] >= overlap:
                            best, overlap = j, float(ious[i, j])
                    if best >= 0:
                        used.add(best)
                        status[a * 10 + t, i] = -1 if ignored[best] else 1
                    elif low <= pa[i] <= high:
                        status[a * 10 + t, i] = 0
    return status, ranks, counts


def accumulate(classes, ranks, status, counts):
    """101-point interpolated precision and recall (instance.py:300-331).

    Inputs are already in global descending score order.
    """
    C = counts.shape[0]
    precision = np.full((10, 101, C, 4, 3), -1.0)
    recall = np.full((10, C, 4, 3), -1.0)
    thresholds = np.arange(101, dtype=np.float64) * 0.01
    eps = np.finfo(np.float64).eps
    for c in range(C):
        for a in range(4):
            if not counts[c, a]:
                continue
            for m, maximum in enumerate(MAX_DETECTIONS):
                selected = (classes == c) & (ranks > 0) & (ranks <= maximum)
                flags = status[a * 10:a * 10 + 10][:, selected]
                n = flags.shape[1]
                if n == 0:
                    precision[:, :, c, a, m] = 0
                    recall[:, c, a, m] = 0
                    continue
                tp = np.cumsum(flags == 1, axis=1).astype(np.float64)
                fp = np.cumsum(flags == 0, axis=1).astype(np.float64)
                rc = tp / counts[c, a]
                pr = tp / (tp + fp + eps)
                envelope = np.maximum.accumulate(pr[:, ::-1], axis=1)[:, ::-1]
                positions = np.stack([np.searchsorted(rc[t], thresholds, side="left") for t in range(10)])
                gathered = np.take_along_axis(envelope, np.minimum(positions, n - 1), 1)
                precision[:, :, c, a, m] = np.where(positions < n, gathered, 0)
                recall[:, c, a, m] = rc[:, -1]
    return precision, recall


def mean_valid(values):
    """Mean of entries >= 0, or -1 when none (instance.py:230-233)."""
    valid = values >= 0
    if not valid.any():
        return np.float64(-1.0)
    return np.where(valid, values, 0).sum() / max(int(valid.sum()), 1)


def summarize(precision, recall):
    """The 12 COCO summaries (instance.py:236-248)."""
    result = {
        "ap": mean_valid(precision[:, :, :, 0, 2]),
        "ap50": mean_valid(precision[0, :, :, 0, 2]),
        "ap75": mean_valid(precision[5, :, :, 0, 2]),
    }
    for area, name in enumerate(("small", "medium", "large"), 1):
        result[f"ap_{name}"] = mean_valid(precision[:, :, :, area, 2])
        result[f"ar_{name}"] = mean_valid(recall[:, :, area, 2])
    for index, maximum in enumerate(MAX_DETECTIONS):
        result[f"ar{maximum}"] = mean_valid(recall[:, :, 0, index])
    result.update(precision=precision, recall=recall)
    return result


def _check_finite(values, name, validate):
    if validate and (not np.isfinite(values).all() or (name == "areas" and (values < 0).any())):
        raise ValueError(f"{name} must be finite; areas must be nonnegative")


class InstanceOracle:
    """Mirror of ``InstanceEvaluator`` on CPU (instance.py:46-227)."""

    def __init__(self, num_classes, validate=True):
        self.num_classes = num_classes
        self.validate = validate
        self.reset()

    def reset(self):
        self.records = []  # (scores, classes, ranks, status) per image
        self.counts = np.zeros((self.num_classes, 4), np.int64)

    def _classes(self, classes):
        classes = np.asarray(classes)
        if self.validate and ((classes < 0) | (classes >= self.num_classes)).any():
            raise ValueError("classes must be valid category indices")
        return classes.astype(np.int32)

    def update(self, pred_masks, pred_classes, pred_scores, gt_masks, gt_classes,
               gt_crowd=None, gt_areas=None):
        """One call per batch; every argument is a list with one array per image."""
        records, counts = [], np.zeros_like(self.counts)
        staged = []
        for b in range(len(pred_masks)):
            pm, gm = np.asarray(pred_masks[b], bool), np.asarray(gt_masks[b], bool)
            pc, gc = self._classes(pred_classes[b]), self._classes(gt_classes[b])
            scores = np.asarray(pred_scores[b], np.float64)
            _check_finite(scores, "scores", self.validate)
            hw = int(np.prod(pm.shape[1:]))
            pa = pm.reshape(len(pm), hw).sum(1).astype(np.float64)
            ga = gm.reshape(len(gm), hw).sum(1).astype(np.float64)
            if self.validate and ((pa == 0).any() or (ga == 0).any()):
                raise ValueError("each instance mask must have pixels")
            crowd = (np.asarray(gt_crowd[b], bool) if gt_crowd is not None
                     else np.zeros(len(gm), bool))
            areas = ga
            if gt_areas is not None:
                areas = np.asarray(gt_areas[b], np.float64)
                _check_finite(areas, "areas", self.validate)
            if pm.shape[1:] != gm.shape[1:]:
                raise ValueError("prediction and target must have matching image counts and dimensions")
            order = score_order(scores)
            staged.append((pm[order], gm, pc[order], gc, pa[order], ga, crowd, areas, scores[order]))
        for pm, gm, pc, gc, pa, ga, crowd, areas, scores in staged:
            ious = mask_ious(pm, gm, pa, ga, crowd)
            status, ranks, positive = match_ious(ious, pc, gc, pa, crowd, areas, self.num_classes)
            records.append((scores, pc, ranks, status))
            counts += positive
        self.records.extend(records)
        self.counts += counts
        return self

    def add_record(self, scores, classes, ranks, status, positive):
        self.records.append((np.asarray(scores, np.float64), np.asarray(classes, np.int32),
                             np.asarray(ranks, np.int32), np.asarray(status, np.int8)))
        self.counts += positive

    def compute(self):
        if self.records:
            scores = np.concatenate([r[0] for r in self.records])
            classes = np.concatenate([r[1] for r in self.records])
            ranks = np.concatenate([r[2] for r in self.records])
            status = np.concatenate([r[3] for r in self.records], axis=1)
            order = score_order(scores)
            classes, ranks, status = classes[order], ranks[order], status[:, order]
        else:
            classes = np.zeros(0, np.int32)
            ranks = np.zeros(0, np.int32)
            status = np.zeros((40, 0), np.int8)
        precision, recall = accumulate(classes, ranks, status, self.counts)
        return summarize(precision, recall)
