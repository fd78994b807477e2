"""Oracle: joint PQ/mIoU + mask AP with one shared panoptic target.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``). Restates
``panoptic_evaluator/combined.py`` (CPU branch).
"""

from __future__ import annotations

import numpy as np

from . import instance as inst
from . import panoptic as pan


def detection_histogram(masks, order, target_map, S):
    """Per detection (in score order), pixel counts of every target slot (combined.py:98-106).

    Pixels on void and stuff count too, so row sums are full detection areas.
    """
    D = len(order)
    pairs = np.zeros((D, S), np.int64)
    flat_target = np.asarray(target_map).reshape(-1).astype(np.int64)
    for rank, index in enumerate(order):
        covered = flat_target[np.asarray(masks[index]).reshape(-1)]
        pairs[rank] = np.bincount(covered, minlength=S)[:S]
    return pairs


def histogram_ious(pairs, pa, ga, crowd):
    """IoU from detection x slot intersections (combined.py:143-150)."""
    inter = pairs.astype(np.float64)
    union = np.where(crowd[None], pa[:, None], pa[:, None] + ga[None] - inter)
    return inter / np.maximum(union, 1)


class SegmentationOracle:
    """Mirror of ``SegmentationEvaluator`` on CPU (combined.py:18-167)."""

    def __init__(self, num_classes, isthing=None, validate=True):
        self.num_classes = num_classes
        self.validate = validate
        self.panoptic = pan.PanopticOracle(num_classes, isthing, validate)
        self.instance = inst.InstanceOracle(num_classes, validate)
        self.isthing = self.panoptic.isthing

    def reset(self):
        self.panoptic.reset()
        self.instance.reset()

    def update(self, pred_map, pred_classes, det_masks, det_classes, det_scores,
               target_map, target_classes, target_crowd=None, instance_areas=None):
        C = self.num_classes
        target_map = np.asarray(target_map)
        classes = np.asarray(target_classes, np.int32)
        crowd = (np.zeros(classes.shape, bool) if target_crowd is None
                 else np.asarray(target_crowd, bool))
        if self.validate:
            pan.validate(target_map, classes, crowd, C)
        if len(det_masks) != len(target_map):
            raise ValueError("detections and target must have matching image counts and dimensions")
        prepared = []
        for b in range(len(det_masks)):
            masks = np.asarray(det_masks[b], bool)
            labels = np.asarray(det_classes[b])
            scores = np.asarray(det_scores[b], np.float64)
            if masks.shape[1:] != target_map.shape[1:]:
                raise ValueError("detections and target must have matching image counts and dimensions")
            if self.validate:
                if not np.isfinite(scores).all():
                    raise ValueError("scores must be finite; areas must be nonnegative")
                if ((labels < 0) | (labels >= C)).any():
                    raise ValueError("classes must be valid category indices")
            order = inst.score_order(scores)
            prepared.append((masks, labels[order].astype(np.int32), scores[order], order))
        if instance_areas is not None:
            instance_areas = np.asarray(instance_areas, np.float64)
            if instance_areas.shape != classes.shape:
                raise ValueError("instance_areas must be floating point B x S on evaluator device")
            if self.validate and (not np.isfinite(instance_areas).all() or (instance_areas < 0).any()):
                raise ValueError("instance_areas must be finite and nonnegative")
        histograms, detection_areas = [], []
        S = classes.shape[1]
        for (masks, labels, scores, order), tmap in zip(prepared, target_map):
            if self.validate and (~self.isthing[labels.astype(np.int64)]).any():
                raise ValueError("detection categories must be thing classes")
            pairs = detection_histogram(masks, order, tmap, S)
            areas = pairs.sum(1).astype(np.float64)
            if self.validate and (areas == 0).any():
                raise ValueError("each instance mask must have pixels")
            histograms.append(pairs)
            detection_areas.append(areas)
        target_areas = self.panoptic.update(pred_map, pred_classes, target_map, classes, crowd,
                                            return_areas=True)
        valid_classes = np.clip(classes, 0, C - 1).astype(np.int64)
        gt_classes = np.where((classes >= 0) & self.isthing[valid_classes], classes, -1).astype(np.int32)
        for b, ((masks, labels, scores, order), pairs, pa) in enumerate(
                zip(prepared, histograms, detection_areas)):
            ga = target_areas[b].astype(np.float64)
            annotation = ga if instance_areas is None else instance_areas[b]
            ious = histogram_ious(pairs, pa, ga, crowd[b])
            status, ranks, positive = inst.match_ious(ious, labels, gt_classes[b], pa, crowd[b],
                                                      annotation, C)
            self.instance.add_record(scores, labels, ranks, status, positive)
        return self

    def compute(self):
        result = self.panoptic.compute()
        result["instance"] = self.instance.compute()
        return result


def image_update(args):
    """One image through a fresh oracle (picklable; used by the CPU baseline's process pool)."""
    (pred_map, pred_classes, det_masks, det_classes, det_scores, target_map, target_classes, crowd,
     num_classes, isthing) = args
    oracle = SegmentationOracle(num_classes, isthing, validate=False)
    oracle.update(pred_map[None], pred_classes[None], [det_masks], [det_classes], [det_scores], target_map[None],
                  target_classes[None], crowd[None])
    return oracle


def merge(oracles, num_classes, isthing):
    """Sum per-image oracle states in order (integer sums exact; records concatenated)."""
    total = SegmentationOracle(num_classes, isthing, validate=False)
    for o in oracles:
        for name in ("tp", "fp", "fn", "iou_sum", "confusion"):
            setattr(total.panoptic, name, getattr(total.panoptic, name) + getattr(o.panoptic, name))
        total.instance.records.extend(o.instance.records)
        total.instance.counts += o.instance.counts
    return total
