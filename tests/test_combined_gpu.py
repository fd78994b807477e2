"""GPU parity of SegmentationEvaluator (reference tests/test_combined.py) against golden vectors and the oracle."""

import numpy as np
import pytest
import torch

from golden_io import load
from helpers import assert_tree, cuda
from oracle import combined as ocomb

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pe():
    import panoptic_evaluator_gb300 as pe
    return pe


def fixture(pe):
    inputs, expected = load("combined")
    target = pe.PanopticBatch(cuda(inputs["maps"]), cuda(inputs["classes"]), cuda(inputs["crowd"]))
    prediction = pe.PanopticBatch(cuda(inputs["pred_maps"]), cuda(inputs["classes"]))
    detections = pe.InstanceBatch([cuda(m) for m in inputs["masks"]], [cuda(c) for c in inputs["labels"]],
                                  [cuda(s) for s in inputs["scores"]])
    return inputs, expected, prediction, detections, target


def instance_target(pe, target, areas=None):
    masks, classes, crowd, ann = [], [], [], []
    for b in range(len(target.segment_map)):
        slots = torch.where((target.classes[b] >= 0) & (target.classes[b] < 2))[0]
        masks.append(target.segment_map[b][None] == slots[:, None, None])
        classes.append(target.classes[b, slots])
        crowd.append(target.crowd[b, slots])
        if areas is not None:
            ann.append(areas[b, slots])
    return pe.InstanceBatch(masks, classes, crowd=crowd, areas=ann if areas is not None else None)


def compare(actual, panoptic, instance):
    for key in ("tp", "fp", "fn", "iou_sum", "confusion", "miou"):
        torch.testing.assert_close(actual[key], panoptic[key], rtol=0, atol=1e-14)
    for key in ("All", "Things", "Stuff", "per_class"):
        for metric in panoptic[key]:
            torch.testing.assert_close(actual[key][metric], panoptic[key][metric], rtol=0, atol=1e-14, equal_nan=True)
    for key, value in instance.items():
        torch.testing.assert_close(actual["instance"][key], value, rtol=0, atol=1e-14)


def test_golden_combined(pe):
    inputs, expected, prediction, detections, target = fixture(pe)
    for validate in (True, False):
        joint = pe.SegmentationEvaluator(3, isthing=[True, True, False], validate=validate)
        for areas in (None, cuda(inputs["areas"])):
            joint.update(prediction, detections, target, instance_areas=areas)
        assert_tree(joint.compute(), expected)


def test_separate_evaluator_parity(pe):
    inputs, _, p, d, g = fixture(pe)
    for validate in (True, False):
        joint = pe.SegmentationEvaluator(3, isthing=[True, True, False], validate=validate)
        pq = pe.PanopticEvaluator(3, isthing=[True, True, False], validate=validate)
        ap = pe.InstanceEvaluator(3, validate=validate)
        for areas in (None, cuda(inputs["areas"])):
            joint.update(p, d, g, instance_areas=areas)
            pq.update(p, g)
            ap.update(d, instance_target(pe, g, areas))
        compare(joint.compute(), pq.compute(), ap.compute())
        snapshot = joint.compute()
        joint.reset()
        assert joint.compute()["instance"]["ap"].item() == -1.0
        compare(snapshot, pq.compute(), ap.compute())


def test_original_ids_and_empty_detections(pe):
    _, _, p, d, g = fixture(pe)
    original = g.segment_map.long() * 10000000001
    info = [[dict(id=int(slot) * 10000000001, category_id=int(g.classes[b, slot]), iscrowd=int(g.crowd[b, slot]))
             for slot in range(1, g.classes.shape[1]) if g.classes[b, slot] >= 0] for b in range(2)]
    target = pe.PanopticBatch.from_coco(original, info, [0, 1, 2], compact=False)
    empty = pe.InstanceBatch([torch.empty((0, 13, 35), dtype=torch.bool, device="cuda") for _ in range(2)],
                             [torch.empty(0, dtype=torch.int32, device="cuda") for _ in range(2)],
                             [torch.empty(0, device="cuda") for _ in range(2)])
    joint = pe.SegmentationEvaluator(3, isthing=[True, True, False])
    joint.update(p, empty, target)
    pq = pe.PanopticEvaluator(3, isthing=[True, True, False])
    pq.update(p, g)
    ap = pe.InstanceEvaluator(3)
    ap.update(empty, instance_target(pe, g))
    compare(joint.compute(), pq.compute(), ap.compute())


def test_failed_validation_preserves_all_metrics(pe):
    _, _, p, d, g = fixture(pe)
    joint = pe.SegmentationEvaluator(3, isthing=[True, True, False])
    joint.update(p, d, g)
    before = joint.compute()
    labels = [x.clone() for x in d.classes]
    labels[1][-1] = 2
    with pytest.raises(ValueError, match="thing"):
        joint.update(p, pe.InstanceBatch(d.masks, labels, d.scores), g)
    masks = [x.clone() for x in d.masks]
    masks[1][-1].zero_()
    with pytest.raises(ValueError, match="pixels"):
        joint.update(p, pe.InstanceBatch(masks, d.classes, d.scores), g)
    with pytest.raises(ValueError, match="instance_areas"):
        joint.update(p, d, g, instance_areas=torch.full(g.classes.shape, float("nan"), device="cuda"))
    compare(joint.compute(), before, before["instance"])


def test_nondefault_stream_and_snapshot(pe):
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        _, _, p, d, g = fixture(pe)
        joint = pe.SegmentationEvaluator(3, isthing=[True, True, False], validate=False)
        pq = pe.PanopticEvaluator(3, isthing=[True, True, False], validate=False)
        ap = pe.InstanceEvaluator(3, validate=False)
        pq.update(p, g)
        ap.update(d, instance_target(pe, g))
        joint.update(p, d, g)
        actual, expected_pq, expected_ap = joint.compute(), pq.compute(), ap.compute()
        g.segment_map.zero_()
        for x in d.masks + d.scores:
            x.zero_()
        joint.reset()
    stream.synchronize()
    compare(actual, expected_pq, expected_ap)


@pytest.mark.parametrize("seed,hw", [(0, (120, 176)), (1, (120, 176)), (2, (97, 131)), (3, (33, 47))])
def test_config_shaped_batch_against_oracle(pe, seed, hw):
    """Rows of H x W bytes: a multiple of 16 (aligned) or odd (every mask row at another offset)."""
    from panoptic_evaluator_gb300 import synthetic
    images = synthetic.segmentation_batch(seed=seed, images=3, fixed_hw=hw, fixed_slots=40, dets=(5, 30))
    C = 133
    isthing = list(np.arange(C) < 80)
    P = max(len(i.pred_classes) for i in images)
    pad = lambda a, n: np.pad(a, (0, n - len(a)), constant_values=-1)  # noqa: E731
    oracle = ocomb.SegmentationOracle(C, isthing)
    oracle.update(np.stack([i.pred for i in images]), np.stack([pad(i.pred_classes, P) for i in images]),
                  [i.det_masks for i in images], [i.det_classes for i in images], [i.scores for i in images],
                  np.stack([i.target for i in images]), np.stack([i.target_classes for i in images]),
                  np.stack([i.crowd for i in images]))
    joint = pe.SegmentationEvaluator(C, isthing=isthing)
    joint.update(pe.PanopticBatch(cuda(np.stack([i.pred for i in images])),
                                  cuda(np.stack([pad(i.pred_classes, P) for i in images]))),
                 pe.InstanceBatch([cuda(i.det_masks) for i in images], [cuda(i.det_classes) for i in images],
                                  [cuda(i.scores) for i in images]),
                 pe.PanopticBatch(cuda(np.stack([i.target for i in images])),
                                  cuda(np.stack([i.target_classes for i in images])),
                                  cuda(np.stack([i.crowd for i in images]))))
    assert_tree(joint.compute(), oracle.compute())


@pytest.mark.parametrize("dynamic,bulk", [(True, True), (False, True), (False, False)])
def test_chunk_schedules_give_identical_results(pe, monkeypatch, dynamic, bulk):
    """Chunks from the device counter, host ranges of equal bytes, or the register-load pass: same counts."""
    from panoptic_evaluator_gb300 import combined, synthetic
    from panoptic_evaluator_gb300.ragged import SegmentationImages
    monkeypatch.setattr(combined, "DYNAMIC_PASS", dynamic)
    monkeypatch.setattr(combined, "BULK_PASS", bulk)
    images = synthetic.segmentation_batch(seed=41, images=24, side=(60, 300), slots=(5, 60), dets=(0, 40))
    C = 133
    isthing = list(np.arange(C) < 80)
    oracle = ocomb.SegmentationOracle(C, isthing)
    for i in images:
        oracle.update(i.pred[None], i.pred_classes[None], [i.det_masks], [i.det_classes], [i.scores], i.target[None],
                      i.target_classes[None], i.crowd[None])
    arena = SegmentationImages([i.target for i in images], [i.target_classes for i in images],
                               [i.crowd for i in images], [i.pred for i in images], [i.pred_classes for i in images],
                               [i.det_masks for i in images], [i.det_classes for i in images],
                               [i.scores for i in images])
    joint = pe.SegmentationEvaluator(C, isthing=isthing)
    joint.update_images(arena)
    assert_tree(joint.compute(), oracle.compute())


def test_grid_workload_against_oracle(pe):
    """The grid-shaped workload of the recorded reference timings, small: same results as the oracle."""
    from panoptic_evaluator_gb300 import synthetic
    images, things = synthetic.grid_batch(seed=5, images=3, height=48, width=72, segments=16, detections=20)
    oracle = ocomb.SegmentationOracle(15, things)
    oracle.update(np.stack([i.pred for i in images]), np.stack([i.pred_classes for i in images]),
                  [i.det_masks for i in images], [i.det_classes for i in images], [i.scores for i in images],
                  np.stack([i.target for i in images]), np.stack([i.target_classes for i in images]),
                  np.stack([i.crowd for i in images]))
    joint = pe.SegmentationEvaluator(15, isthing=things)
    joint.update(pe.PanopticBatch(cuda(np.stack([i.pred for i in images])),
                                  cuda(np.stack([i.pred_classes for i in images]))),
                 pe.InstanceBatch([cuda(i.det_masks) for i in images], [cuda(i.det_classes) for i in images],
                                  [cuda(i.scores) for i in images]),
                 pe.PanopticBatch(cuda(np.stack([i.target for i in images])),
                                  cuda(np.stack([i.target_classes for i in images])),
                                  cuda(np.stack([i.crowd for i in images]))))
    assert_tree(joint.compute(), oracle.compute())


def test_large_histograms_scored_in_place(pe):
    """220 target x 240 prediction slots per image: histograms too large to stage, scored in place."""
    from panoptic_evaluator_gb300 import synthetic
    images = synthetic.segmentation_batch(seed=7, images=3, fixed_hw=(64, 96), fixed_slots=220, dets=(3, 12))
    P = max(len(i.pred_classes) for i in images)
    assert len(images[0].target_classes) * P * 4 > 100 * 1024  # past the 100 KB staging limit
    C = 133
    isthing = list(np.arange(C) < 80)
    pad = lambda a, n: np.pad(a, (0, n - len(a)), constant_values=-1)  # noqa: E731
    oracle = ocomb.SegmentationOracle(C, isthing)
    oracle.update(np.stack([i.pred for i in images]), np.stack([pad(i.pred_classes, P) for i in images]),
                  [i.det_masks for i in images], [i.det_classes for i in images], [i.scores for i in images],
                  np.stack([i.target for i in images]), np.stack([i.target_classes for i in images]),
                  np.stack([i.crowd for i in images]))
    joint = pe.SegmentationEvaluator(C, isthing=isthing)
    joint.update(pe.PanopticBatch(cuda(np.stack([i.pred for i in images])),
                                  cuda(np.stack([pad(i.pred_classes, P) for i in images]))),
                 pe.InstanceBatch([cuda(i.det_masks) for i in images], [cuda(i.det_classes) for i in images],
                                  [cuda(i.scores) for i in images]),
                 pe.PanopticBatch(cuda(np.stack([i.target for i in images])),
                                  cuda(np.stack([i.target_classes for i in images])),
                                  cuda(np.stack([i.crowd for i in images]))))
    assert_tree(joint.compute(), oracle.compute())
