"""Seeded synthetic workloads with COCO-like shapes (no dataset items are used).

Five generators, one per benchmark workload:

* ``voronoi_batch``      8 x 256 x 256 maps, 24 Voronoi segments, 20 classes.
* ``coco_panoptic_batch`` B x 640 x 640 padded maps: stuff Voronoi regions plus
  5-60 thing ellipses (log-uniform 32-20000 px), 133 classes.
* ``instance_batch``     per-image bool ellipse masks (gt 1-50, 100 predictions,
  70 % perturbed copies of gt), Beta-distributed scores, 80 classes.
* ``segmentation_batch`` uneven images (sides 320-1024) with a panoptic target,
  a perturbed panoptic prediction and detections cut from the target's thing
  segments.
* ``prefix_sequence``    a generation-ordered mask sequence for one target.

Everything is numpy on the host so a seed gives the same arrays on every
machine. Metadata is always consistent with the maps (active slots have
pixels), so validation passes.
"""

from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

COCO_THINGS, COCO_STUFF = 80, 53


def _nearest_site(h, w, sites):
    yy, xx = np.mgrid[0:h, 0:w]
    points = np.stack((yy.ravel(), xx.ravel()), 1).astype(np.float32)
    best = np.zeros(points.shape[0], np.int32)
    best_d = np.full(points.shape[0], np.inf, np.float32)
    for i, (sy, sx) in enumerate(sites):
        d = (points[:, 0] - sy) ** 2 + (points[:, 1] - sx) ** 2
        closer = d < best_d
        best[closer] = i
        best_d[closer] = d[closer]
    return best.reshape(h, w)


def _ellipse(rng, h, w, area):
    """Boolean crop and offset of a random rotated ellipse of about `area` pixels."""
    ratio = rng.uniform(0.5, 2.0)
    a = math.sqrt(area / math.pi * ratio)
    b = math.sqrt(area / math.pi / ratio)
    theta = rng.uniform(0, math.pi)
    r = int(math.ceil(max(a, b))) + 1
    cy, cx = rng.uniform(0, h), rng.uniform(0, w)
    y0, y1 = max(0, int(cy) - r), min(h, int(cy) + r + 1)
    x0, x1 = max(0, int(cx) - r), min(w, int(cx) + r + 1)
    yy, xx = np.mgrid[y0:y1, x0:x1]
    dy, dx = yy - cy, xx - cx
    c, s = math.cos(theta), math.sin(theta)
    u, v = (dx * c + dy * s) / a, (-dx * s + dy * c) / b
    return (u * u + v * v) <= 1.0, (y0, x0)


def _neighbour_relabel(rng, labels, fraction):
    h, w = labels.shape
    out = labels.copy()
    n = int(fraction * h * w)
    ys, xs = rng.integers(0, h, n), rng.integers(0, w, n)
    direction = rng.integers(0, 4, n)
    ny = np.clip(ys + np.array([-1, 1, 0, 0])[direction], 0, h - 1)
    nx = np.clip(xs + np.array([0, 0, -1, 1])[direction], 0, w - 1)
    out[ys, xs] = labels[ny, nx]
    return out


def _perturb_prediction(rng, target, slot_classes, num_classes, capacity, *, split=0.05, merge=0.03,
                        flip=0.1, relabel=0.1, spurious=0, thing_classes=None, image_hw=None):
    """Jitter boundaries, split / merge segments, flip classes, add spurious segments.

    Returns (pred map, pred classes [capacity]) with consistent metadata.
    """
    h, w = target.shape
    pred = _neighbour_relabel(rng, target, relabel)
    pred[target == 0] = 0  # keep padding void
    classes = np.full(capacity, -1, np.int64)
    present = np.unique(pred)
    present = present[present > 0]
    next_slot = int(present.max()) + 1 if present.size else 1
    for s in present:
        classes[s] = slot_classes[s]
    segments = list(present)
    # Splits: a half-plane through the segment centroid gets a new slot.
    for s in segments:
        if rng.random() < split and next_slot < capacity:
            ys, xs = np.nonzero(pred == s)
            if ys.size < 2:
                continue
            angle = rng.uniform(0, 2 * math.pi)
            side = (ys - ys.mean()) * math.cos(angle) + (xs - xs.mean()) * math.sin(angle) > 0
            if side.any() and (~side).any():
                pred[ys[side], xs[side]] = next_slot
                classes[next_slot] = classes[s]
                next_slot += 1
    # Merges: a segment takes the slot of a random neighbour.
    for s in segments:
        if rng.random() < merge:
            ys, xs = np.nonzero(pred == s)
            if ys.size == 0:
                continue
            i = rng.integers(0, ys.size)
            for dy, dx in ((1, 0), (-1, 0), (0, 1), (0, -1)):
                y, x = ys[i] + dy, xs[i] + dx
                if 0 <= y < h and 0 <= x < w and pred[y, x] not in (0, s):
                    pred[pred == s] = pred[y, x]
                    break
    for _ in range(spurious):
        if next_slot >= capacity:
            break
        hh, ww = image_hw if image_hw is not None else (h, w)
        mask, (y0, x0) = _ellipse(rng, hh, ww, math.exp(rng.uniform(math.log(32), math.log(20000))))
        sub = pred[y0:y0 + mask.shape[0], x0:x0 + mask.shape[1]]
        sub[mask] = next_slot
        classes[next_slot] = rng.integers(0, thing_classes or num_classes)
        next_slot += 1
    flip_mask = rng.random(capacity) < flip
    classes = np.where(flip_mask & (classes >= 0), rng.integers(0, num_classes, capacity), classes)
    counts = np.bincount(pred.ravel(), minlength=capacity)[:capacity]
    classes[counts == 0] = -1
    classes[0] = -1
    return pred.astype(np.int32), classes.astype(np.int32)


@dataclass
class PanopticArrays:
    gt: np.ndarray  # B x H x W int32
    gc: np.ndarray  # B x G int32
    crowd: np.ndarray  # B x G bool
    pred: np.ndarray  # B x H x W int32
    pc: np.ndarray  # B x P int32
    num_classes: int
    isthing: np.ndarray  # C bool


def voronoi_batch(seed=0, B=8, H=256, W=256, sites=24, S=32, num_classes=20, things=12) -> PanopticArrays:
    """Voronoi target of `sites` segments with 2 % crowd things and 5 % void pixels."""
    rng = np.random.default_rng(seed)
    gt = np.zeros((B, H, W), np.int32)
    pred = np.zeros_like(gt)
    gc = np.full((B, S), -1, np.int32)
    pc = np.full((B, S), -1, np.int32)
    crowd = np.zeros((B, S), bool)
    for b in range(B):
        points = rng.uniform((0, 0), (H, W), (sites, 2))
        target = _nearest_site(H, W, points) + 1
        target[rng.random((H, W)) < 0.05] = 0
        slot_classes = np.full(S, -1, np.int64)
        slot_classes[1:sites + 1] = rng.integers(0, num_classes, sites)
        counts = np.bincount(target.ravel(), minlength=S)
        slot_classes[counts == 0] = -1
        slot_classes[0] = -1
        gt[b] = target
        gc[b] = slot_classes
        crowd[b] = (slot_classes >= 0) & (slot_classes < things) & (rng.random(S) < 0.02)
        pred[b], pc[b] = _perturb_prediction(rng, target, slot_classes, num_classes, S)
    isthing = np.arange(num_classes) < things
    return PanopticArrays(gt, gc, crowd, pred, pc, num_classes, isthing)


def _coco_target(rng, H, W, canvas_h, canvas_w, G, num_classes, things, max_things=60):
    target = np.zeros((canvas_h, canvas_w), np.int32)
    classes = np.full(G, -1, np.int64)
    if G < 2:
        raise ValueError("a COCO-like target needs at least two slots (void and one segment)")
    # 3-8 stuff segments, at most G - 1 (the same draw whenever G >= 10)
    n_stuff = int(rng.integers(3, 9)) if G >= 10 else int(rng.integers(min(3, G - 1), G))
    points = rng.uniform((0, 0), (H, W), (n_stuff, 2))
    target[:H, :W] = _nearest_site(H, W, points) + 1
    classes[1:n_stuff + 1] = things + rng.integers(0, num_classes - things, n_stuff)
    slot = n_stuff + 1
    n_things = int(rng.integers(5, max_things + 1))
    for _ in range(n_things):
        if slot >= G:
            break
        area = math.exp(rng.uniform(math.log(32), math.log(20000)))
        mask, (y0, x0) = _ellipse(rng, H, W, area)
        target[y0:y0 + mask.shape[0], x0:x0 + mask.shape[1]][mask] = slot
        classes[slot] = rng.integers(0, things)
        slot += 1
    counts = np.bincount(target.ravel(), minlength=G)[:G]
    classes[counts == 0] = -1
    classes[0] = -1
    return target, classes


def coco_panoptic_batch(seed=1, B=16, canvas=640, side=(480, 640), G=101, P=121,
                        num_classes=COCO_THINGS + COCO_STUFF, things=COCO_THINGS) -> PanopticArrays:
    """COCO-shaped panoptic batch on a padded canvas (void outside each image)."""
    rng = np.random.default_rng(seed)
    gt = np.zeros((B, canvas, canvas), np.int32)
    pred = np.zeros_like(gt)
    gc = np.full((B, G), -1, np.int32)
    pc = np.full((B, P), -1, np.int32)
    crowd = np.zeros((B, G), bool)
    for b in range(B):
        H, W = (int(v) for v in rng.integers(side[0], side[1] + 1, 2))
        target, classes = _coco_target(rng, H, W, canvas, canvas, G, num_classes, things)
        gt[b], gc[b] = target, classes
        crowd[b] = (classes >= 0) & (classes < things) & (rng.random(G) < 0.01)
        spurious = int(0.1 * np.count_nonzero((classes >= 0) & (classes < things)))
        pred[b], pc[b] = _perturb_prediction(rng, target, np.pad(classes, (0, max(0, P - G)), constant_values=-1),
                                             num_classes, P, spurious=spurious, thing_classes=things,
                                             image_hw=(H, W))
    isthing = np.arange(num_classes) < things
    return PanopticArrays(gt, gc, crowd, pred, pc, num_classes, isthing)


def _perturb_mask(rng, mask, shift=8, morph=5):
    """Shift by up to `shift` pixels and dilate / erode by 1..`morph` pixels (bbox-local)."""
    from scipy import ndimage

    h, w = mask.shape
    ys, xs = np.nonzero(mask)
    if ys.size == 0:
        return mask.copy()
    k = int(rng.integers(1, morph + 1))
    dy, dx = (int(v) for v in rng.integers(-shift, shift + 1, 2))
    y0, y1 = max(0, ys.min() - k - 1), min(h, ys.max() + k + 2)
    x0, x1 = max(0, xs.min() - k - 1), min(w, xs.max() + k + 2)
    crop = mask[y0:y1, x0:x1]
    crop = (ndimage.binary_dilation(crop, iterations=k) if rng.random() < 0.5
            else ndimage.binary_erosion(crop, iterations=k))
    if not crop.any():
        crop = mask[y0:y1, x0:x1]
    out = np.zeros_like(mask)
    ty0, tx0 = y0 + dy, x0 + dx
    sy0, sx0 = max(0, -ty0), max(0, -tx0)
    ty0c, tx0c = max(0, ty0), max(0, tx0)
    ty1, tx1 = min(h, y0 + dy + crop.shape[0]), min(w, x0 + dx + crop.shape[1])
    if ty1 > ty0c and tx1 > tx0c:
        out[ty0c:ty1, tx0c:tx1] = crop[sy0:sy0 + ty1 - ty0c, sx0:sx0 + tx1 - tx0c]
    if not out.any():
        out = mask.copy()
    return out


def _ellipse_mask(rng, h, w, area):
    mask = np.zeros((h, w), bool)
    crop, (y0, x0) = _ellipse(rng, h, w, area)
    mask[y0:y0 + crop.shape[0], x0:x0 + crop.shape[1]] = crop
    if not mask.any():
        mask[int(rng.integers(0, h)), int(rng.integers(0, w))] = True
    return mask


@dataclass
class InstanceImage:
    pred_masks: np.ndarray  # D x H x W bool
    pred_classes: np.ndarray  # D int64
    scores: np.ndarray  # D float32
    gt_masks: np.ndarray  # G x H x W bool
    gt_classes: np.ndarray  # G int64
    crowd: np.ndarray  # G bool


def instance_one(seed, index, **kwargs) -> InstanceImage:
    """Image `index` of a COCO-like instance batch with its own seeded stream (for parallel generation)."""
    return instance_batch(seed=[seed, index], images=1, **kwargs)[0]


def instance_batch(seed=2, images=32, side=(480, 640), num_classes=COCO_THINGS, gt_range=(1, 50), preds=100,
                   copies=0.7) -> list[InstanceImage]:
    """COCO-like instance masks: ellipse GT, perturbed copies and random ellipses as predictions."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(images):
        h, w = (int(v) for v in rng.integers(side[0], side[1] + 1, 2))
        g = int(rng.integers(gt_range[0], gt_range[1] + 1))
        gt = np.stack([_ellipse_mask(rng, h, w, math.exp(rng.uniform(math.log(32), math.log(20000))))
                       for _ in range(g)])
        gc = rng.integers(0, num_classes, g)
        crowd = rng.random(g) < 0.02
        n_copy = int(round(preds * copies))
        masks, classes, scores = [], [], []
        for i in range(preds):
            if i < n_copy:
                j = int(rng.integers(0, g))
                masks.append(_perturb_mask(rng, gt[j]))
                classes.append(gc[j] if rng.random() > 0.1 else rng.integers(0, num_classes))
                scores.append(rng.beta(5, 2))
            else:
                masks.append(_ellipse_mask(rng, h, w, math.exp(rng.uniform(math.log(32), math.log(20000)))))
                classes.append(rng.integers(0, num_classes))
                scores.append(rng.beta(2, 5))
        out.append(InstanceImage(np.stack(masks), np.array(classes, np.int64), np.array(scores, np.float32),
                                 gt, gc.astype(np.int64), crowd))
    return out


@dataclass
class SegmentationImage:
    target: np.ndarray  # H x W int32 slot map
    target_classes: np.ndarray  # G int32
    crowd: np.ndarray  # G bool
    pred: np.ndarray  # H x W int32
    pred_classes: np.ndarray  # P int32
    det_masks: np.ndarray  # D x H x W bool
    det_classes: np.ndarray  # D int64
    scores: np.ndarray  # D float32


def segmentation_image(rng, h, w, slots, dets, num_classes=COCO_THINGS + COCO_STUFF, things=COCO_THINGS,
                       pred_slots=None) -> SegmentationImage:
    """One image: target with `slots` slots, perturbed prediction, detections cut from thing segments."""
    max_things = max(5, slots - 9)
    target, classes = _coco_target(rng, h, w, h, w, slots, num_classes, things, max_things=max_things)
    crowd = (classes >= 0) & (classes < things) & (rng.random(slots) < 0.01)
    P = pred_slots or slots + 20
    spurious = int(0.1 * np.count_nonzero((classes >= 0) & (classes < things)))
    pred, pc = _perturb_prediction(rng, target, np.pad(classes, (0, P - slots), constant_values=-1), num_classes, P,
                                   spurious=spurious, thing_classes=things)
    thing_slots = np.nonzero((classes >= 0) & (classes < things))[0]
    masks, det_classes, scores = [], [], []
    for _ in range(dets):
        if thing_slots.size and rng.random() < 0.85:
            s = int(rng.choice(thing_slots))
            masks.append(_perturb_mask(rng, target == s))
            det_classes.append(classes[s])
            scores.append(rng.beta(5, 2))
        else:
            masks.append(_ellipse_mask(rng, h, w, math.exp(rng.uniform(math.log(32), math.log(20000)))))
            det_classes.append(rng.integers(0, things))
            scores.append(rng.beta(2, 5))
    return SegmentationImage(target.astype(np.int32), classes.astype(np.int32), crowd, pred, pc,
                             np.stack(masks) if masks else np.zeros((0, h, w), bool),
                             np.array(det_classes, np.int64), np.array(scores, np.float32))


def segmentation_one(seed, index, side=(320, 1024), slots=(10, 150), dets=(5, 100), fixed_hw=None,
                     fixed_slots=None) -> SegmentationImage:
    """Image `index` of a segmentation batch; each image has its own seeded stream."""
    rng = np.random.default_rng([seed, index])
    h, w = fixed_hw or tuple(int(v) for v in rng.integers(side[0], side[1] + 1, 2))
    s = fixed_slots or int(rng.integers(slots[0], slots[1] + 1))
    n = int(rng.integers(dets[0], dets[1] + 1))
    return segmentation_image(rng, h, w, s, n)


def segmentation_batch(seed=3, images=256, side=(320, 1024), slots=(10, 150), dets=(5, 100), fixed_hw=None,
                       fixed_slots=None, pool=None) -> list[SegmentationImage]:
    """Uneven images for the combined evaluator; fixed_hw / fixed_slots give a same-shape batch.

    `pool` (a multiprocessing pool) generates images in parallel with identical results.
    """
    from functools import partial
    make = partial(segmentation_one, seed, side=side, slots=slots, dets=dets, fixed_hw=fixed_hw,
                   fixed_slots=fixed_slots)
    if pool is not None:
        return pool.map(make, range(images), chunksize=max(1, images // 64))
    return [make(i) for i in range(images)]


@dataclass
class PrefixImage:
    target: np.ndarray  # H x W int32
    target_classes: np.ndarray  # G int32
    crowd: np.ndarray  # G bool
    masks: np.ndarray  # N x H x W bool, generation order
    classes: np.ndarray  # N int32


def prefix_one(seed, index, side=(256, 1024), masks=64, slots=101, num_classes=COCO_THINGS + COCO_STUFF,
               things=COCO_THINGS, fixed_hw=None) -> PrefixImage:
    """A generation-ordered mask sequence for one COCO-like target (H x W = fixed_hw, or sides drawn from `side`)."""
    rng = np.random.default_rng([seed, index])
    h, w = fixed_hw if fixed_hw else (int(v) for v in rng.integers(side[0], side[1] + 1, 2))
    target, classes = _coco_target(rng, h, w, h, w, slots, num_classes, things)
    crowd = (classes >= 0) & (classes < things) & (rng.random(slots) < 0.01)
    present = np.nonzero(classes >= 0)[0]
    out, labels = [], []
    for _ in range(masks):
        if present.size and rng.random() < 0.8:
            s = int(rng.choice(present))
            out.append(_perturb_mask(rng, target == s, shift=4, morph=3))
            labels.append(classes[s] if rng.random() > 0.1 else rng.integers(0, num_classes))
        else:
            out.append(_ellipse_mask(rng, h, w, math.exp(rng.uniform(math.log(32), math.log(20000)))))
            labels.append(rng.integers(0, num_classes))
    return PrefixImage(target.astype(np.int32), classes.astype(np.int32), crowd, np.stack(out),
                       np.array(labels, np.int32))


def prefix_batch(seed=5, images=8, side=(256, 1024), masks=64, pool=None) -> list[PrefixImage]:
    """Same-size prefix requests (the side is drawn once) so they batch as B x H x W."""
    from functools import partial
    rng = np.random.default_rng(seed)
    h = int(rng.integers(side[0], side[1] + 1))
    make = partial(prefix_one, seed, side=(h, h), masks=masks)
    return pool.map(make, range(images)) if pool is not None else [make(i) for i in range(images)]


def _dilate5(mask: np.ndarray) -> np.ndarray:
    """5 x 5 binary dilation of a bool H x W mask (separable OR of shifted copies)."""
    h, w = mask.shape
    p = np.pad(mask, 2)
    cols = p[:, 0:w] | p[:, 1:w + 1] | p[:, 2:w + 2] | p[:, 3:w + 3] | p[:, 4:w + 4]
    return cols[0:h] | cols[1:h + 1] | cols[2:h + 2] | cols[3:h + 3] | cols[4:h + 4]


def grid_batch(seed=24, images=8, height=256, width=384, segments=64, detections=64, num_classes=15):
    """The workload shape of the reference's recorded combined timings (A100, 8 images, 15 classes).

    Targets tile each image with a grid of `segments` rectangular cells (slot s in row-major cell
    s - 1 of a ceil(sqrt(segments)) square grid); labels are uniform over the classes (slot 1 is
    class 0, a thing; the first two thirds of the classes are things), 10 % of the slots crowd.
    The prediction is the target with its first three rows void. Detections are 5 x 5 dilations
    of thing targets drawn with replacement (so they reach into their neighbours and overlap),
    with uniform scores. Returns SegmentationImage records plus the thing flags.
    """
    rng = np.random.default_rng(seed)
    side = int(np.ceil(np.sqrt(segments)))
    things = np.arange(num_classes) < max(1, num_classes * 2 // 3)
    rows = np.minimum(np.arange(height) * side // height, side - 1)
    cols = np.minimum(np.arange(width) * side // width, side - 1)
    cell = rows[:, None] * side + cols[None, :]
    target = np.where(cell < segments, cell + 1, 0).astype(np.int32)
    out = []
    for _ in range(images):
        labels = rng.integers(0, num_classes, segments + 1).astype(np.int32)
        labels[0], labels[1] = -1, 0
        crowd = rng.random(segments + 1) < 0.1
        crowd[0] = False
        pred = target.copy()
        pred[:3] = 0
        slots = np.flatnonzero((labels >= 0) & things[np.maximum(labels, 0)])
        picked = rng.integers(0, len(slots), detections)
        dilated = {int(s): _dilate5(target == s) for s in np.unique(slots[picked])}
        masks = np.stack([dilated[int(slots[i])] for i in picked]) if detections else np.zeros((0, height, width), bool)
        out.append(SegmentationImage(target=target.copy(), target_classes=labels, crowd=crowd, pred=pred,
                                     pred_classes=labels.copy(), det_masks=masks,
                                     det_classes=labels[slots[picked]].astype(np.int64),
                                     scores=rng.random(detections).astype(np.float32)))
    return out, list(things)
