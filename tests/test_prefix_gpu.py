"""GPU parity of segmentation_prefixes (reference tests/test_prefix.py) against golden vectors and the oracle."""

import numpy as np
import pytest
import torch

from golden_io import load, scalar
from helpers import assert_tree, cuda
from oracle import prefix as opre

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pe():
    import panoptic_evaluator_gb300 as pe
    return pe


def target(pe):
    return pe.PanopticBatch(torch.tensor([[[1, 1, 2, 2, 3, 0]]], dtype=torch.int32, device="cuda"),
                            torch.tensor([[-1, 0, 0, 1]], dtype=torch.int32, device="cuda"))


def compare_snapshots(actual, expected):
    assert len(actual) == len(expected)
    for a, e in zip(actual, expected):
        assert len(a) == len(e)
        for got, want in zip(a, e):
            assert got["prefix"] == scalar(want["prefix"])
            assert_tree(got, {k: v for k, v in want.items() if k != "prefix"})


def test_golden_prefix_cases(pe):
    cases, outputs = load("prefix")
    for case, expected in zip(cases, outputs):
        checkpoints = None if case["checkpoints"] is None else [int(k) for k in case["checkpoints"]]
        result = pe.segmentation_prefixes(
            pe.InstanceBatch([cuda(case["masks"])], [cuda(case["classes"])]),
            pe.PanopticBatch(cuda(case["maps"]), cuda(case["labels"]), cuda(case["crowd"])), 3,
            isthing=[True, False, True], checkpoints=checkpoints, iou_thresholds=tuple(case["thresholds"].tolist()))
        compare_snapshots(result, expected)


def test_every_prefix_matches_canvas_evaluation(pe):
    t = target(pe)
    g = np.random.default_rng(17)
    for _ in range(5):
        masks = torch.from_numpy(g.random((7, 1, 6)) > .4).cuda()
        masks[:, :, 0] = True
        classes = torch.from_numpy(g.integers(0, 2, 7).astype(np.int32)).cuda()
        actual = pe.segmentation_prefixes(pe.InstanceBatch([masks], [classes]), t, 3, isthing=[True, False, True],
                                          checkpoints=list(range(8)))[0]
        canvas = torch.zeros_like(t.segment_map)
        for k, result in enumerate(actual):
            if k:
                canvas[0][masks[k - 1]] = k
            labels = torch.cat((classes.new_tensor([-1]), classes))
            present = torch.bincount(canvas.flatten().long(), minlength=8) > 0
            labels = torch.where(present, labels, -1)
            ev = pe.PanopticEvaluator(3, isthing=[True, False, True])
            ev.update(pe.PanopticBatch(canvas.clone(), labels[None].contiguous()), t)
            expected = ev.compute()
            for key in ("tp", "fp", "fn", "iou_sum", "confusion", "miou"):
                torch.testing.assert_close(result[key], expected[key], equal_nan=True)
            for key in ("All", "Things", "Stuff", "per_class"):
                for metric in expected[key]:
                    torch.testing.assert_close(result[key][metric], expected[key][metric], equal_nan=True)


def test_independent_masks_duplicates_and_crowd(pe):
    t = target(pe)
    masks = torch.tensor([[[1, 1, 0, 0, 0, 0]], [[1, 1, 0, 0, 0, 0]], [[0, 0, 1, 1, 0, 0]], [[0, 0, 0, 0, 1, 0]]],
                         dtype=torch.bool, device="cuda")
    classes = torch.tensor([0, 0, 0, 1], dtype=torch.int32, device="cuda")
    result = pe.segmentation_prefixes(pe.InstanceBatch([masks], [classes]), t, 2, isthing=[True, False])[0]
    assert [r["instance"]["tp"][0, 0].item() for r in result] == [1, 1, 2, 2]
    assert [r["instance"]["fp"][0, 0].item() for r in result] == [0, 1, 1, 1]
    assert abs(result[-1]["instance"]["precision"][0, 0].item() - 2 / 3) < 1e-15
    crowd = torch.tensor([[False, True, False, False]], device="cuda")
    t2 = pe.PanopticBatch(t.segment_map, t.classes, crowd)
    result = pe.segmentation_prefixes(pe.InstanceBatch([masks], [classes]), t2, 2)[0]
    assert result[1]["instance"]["tp"].sum().item() == 0 and result[1]["instance"]["fp"].sum().item() == 0
    assert result[2]["instance"]["recall"][0, 0].item() == 1


def test_variable_lengths_original_ids_and_thresholds(pe):
    t = target(pe)
    ids = torch.tensor([0, 2**40, 71, 9], device="cuda")
    t = pe.PanopticBatch.from_coco(ids[t.segment_map.long()].repeat(2, 1, 1),
                                   [[dict(id=2**40, category_id=0), dict(id=71, category_id=0),
                                     dict(id=9, category_id=1)]] * 2, [0, 1], compact=False)
    mask = torch.tensor([[[1, 0, 0, 0, 0, 0]]], dtype=torch.bool, device="cuda")
    classes = torch.zeros(1, dtype=torch.int32, device="cuda")
    prediction = pe.InstanceBatch([mask, mask[:0]], [classes, classes[:0]])
    result = pe.segmentation_prefixes(prediction, t, 2)
    assert [r[0]["prefix"] for r in result] == [1, 0]
    assert result[0][0]["instance"]["tp"][:, 0].tolist() == [1, 0]
    assert result[0][0]["instance"]["fp"][:, 0].tolist() == [0, 1]
    selected = pe.segmentation_prefixes(prediction, t, 2, checkpoints=[0])
    assert [r[0]["prefix"] for r in selected] == [0, 0]
    assert pe.segmentation_prefixes(prediction, t, 2, checkpoints=[]) == [[], []]


def test_empty_checkpoints_and_validation(pe):
    t = target(pe)
    prediction = pe.InstanceBatch([torch.empty((0, 1, 6), dtype=torch.bool, device="cuda")],
                                  [torch.empty(0, dtype=torch.int32, device="cuda")])
    result = pe.segmentation_prefixes(prediction, t, 2)[0]
    assert len(result) == 1 and result[0]["prefix"] == 0
    assert result[0]["instance"]["fn"][0].sum().item() == 3
    for kwargs in ({"checkpoints": [1]}, {"checkpoints": [0, 0]}, {"iou_thresholds": [0]},
                   {"iou_thresholds": [float("nan")]}):
        with pytest.raises(ValueError):
            pe.segmentation_prefixes(prediction, t, 2, **kwargs)
    empty_mask = pe.InstanceBatch([torch.zeros((1, 1, 6), dtype=torch.bool, device="cuda")],
                                  [torch.zeros(1, dtype=torch.int32, device="cuda")])
    with pytest.raises(ValueError):
        pe.segmentation_prefixes(empty_mask, t, 2)


@pytest.mark.parametrize("gs,n", [(3, 0), (9, 17), (65, 129), (257, 300)])
def test_cpu_parity_streams_and_snapshots(pe, gs, n):
    g = np.random.default_rng(123 + n)
    maps = g.integers(0, gs, (1, 19, 23)).astype(np.int32)
    maps.reshape(-1)[:gs] = np.arange(gs)
    labels = (np.arange(gs) % 3).astype(np.int32)[None]
    labels[:, 0] = -1
    crowd = g.random((1, gs)) < .3
    crowd[:, 0] = False
    slots = g.integers(1, gs, n) if gs > 1 else np.zeros(0, np.int64)
    masks = maps[0][None] == slots[:, None, None]
    if n:
        masks |= g.random(masks.shape) < .01
    classes = labels[0, slots].astype(np.int32)
    thresholds = (.5,) * 300 if n == 17 else (.5, .75, .95)
    checkpoints = [0, n] if n else [0]
    expected = opre.segmentation_prefixes([masks], [classes], maps, labels, crowd, 3, isthing=[True, False, True],
                                          checkpoints=checkpoints, iou_thresholds=thresholds)
    stream = torch.cuda.Stream()
    stream.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(stream):
        actual = pe.segmentation_prefixes(pe.InstanceBatch([cuda(masks)], [cuda(classes)]),
                                          pe.PanopticBatch(cuda(maps), cuda(labels), cuda(crowd)), 3,
                                          isthing=[True, False, True], checkpoints=checkpoints,
                                          iou_thresholds=thresholds)
    stream.synchronize()
    compare_snapshots(actual, expected)
    # A later call must not mutate retained output storage.
    pe.segmentation_prefixes(pe.InstanceBatch([cuda(masks)], [cuda(classes)]),
                             pe.PanopticBatch(cuda(maps), cuda(labels), cuda(crowd)), 3, isthing=[True, False, True],
                             checkpoints=checkpoints, iou_thresholds=thresholds)
    compare_snapshots(actual, expected)


def test_batched_generation_sequences_against_oracle(pe):
    """Several images with 64 masks each, every 8th prefix and every prefix."""
    from panoptic_evaluator_gb300 import synthetic
    for checkpoints in (list(range(8, 65, 8)), None):
        images = synthetic.prefix_batch(seed=5, images=3, side=(60, 90), masks=64)
        C = 133
        isthing = list(np.arange(C) < 80)
        maps = np.stack([i.target for i in images])
        gc = np.stack([i.target_classes for i in images])
        crowd = np.stack([i.crowd for i in images])
        expected = opre.segmentation_prefixes([i.masks for i in images], [i.classes for i in images], maps, gc, crowd,
                                              C, isthing=isthing, checkpoints=checkpoints)
        actual = pe.segmentation_prefixes(pe.InstanceBatch([cuda(i.masks) for i in images],
                                                           [cuda(i.classes) for i in images]),
                                          pe.PanopticBatch(cuda(maps), cuda(gc), cuda(crowd)), C, isthing=isthing,
                                          checkpoints=checkpoints)
        compare_snapshots(actual, expected)


def test_drop_in_prefix_op(pe):
    from panoptic_evaluator_gb300 import _cuda_evaluator as ce
    t = target(pe)
    masks = torch.tensor([[[1, 1, 0, 0, 0, 0]], [[0, 0, 1, 1, 0, 0]]], dtype=torch.bool, device="cuda")
    classes = torch.tensor([0, 1], dtype=torch.int32, device="cuda")
    outputs = ce.prefix(t.segment_map[0], masks, classes, t.classes[0], torch.zeros(4, dtype=torch.bool, device="cuda"),
                        torch.tensor([True, False], device="cuda"), torch.tensor([0.5, 0.75], dtype=torch.float64,
                                                                                 device="cuda"), [0, 1, 2], True)
    assert len(outputs) == 15 and outputs[-1].item() == 0
    assert tuple(outputs[9].shape) == (3, 2, 2)


def _at_offset(m, offset):
    """Device copy of a bool mask stack whose first byte sits `offset` bytes past an aligned address."""
    flat = torch.zeros(m.size + offset, dtype=torch.bool, device="cuda")
    flat[offset:] = cuda(m).reshape(-1)
    return flat[offset:].view(m.shape)


@pytest.mark.parametrize("h,w,offset", [(32, 48, 0), (64, 64, 0), (64, 64, 3), (33, 47, 0), (33, 47, 9)])
@pytest.mark.parametrize("bulk", [True, False])
def test_aligned_and_unaligned_mask_rows_match_the_oracle(pe, h, w, offset, bulk, monkeypatch):
    """Both owner passes (bulk-copy ring, register loads) on rows that do and do not start 16-byte aligned."""
    from panoptic_evaluator_gb300 import prefix
    monkeypatch.setattr(prefix, "BULK_PASS", bulk)
    g = np.random.default_rng(h * w)
    gs, n = 12, 70
    maps = g.integers(0, gs, (2, h, w)).astype(np.int32)
    maps[:, 0, :gs] = np.arange(gs)
    labels = np.tile((np.arange(gs) % 3).astype(np.int32), (2, 1))
    labels[:, 0] = -1
    crowd = g.random((2, gs)) < 0.2
    crowd[:, 0] = False
    masks, classes = [], []
    for b in range(2):
        slots = g.integers(1, gs, n)
        m = maps[b][None] == slots[:, None, None]
        m |= g.random(m.shape) < 0.02
        masks.append(m)
        classes.append(labels[b, slots].astype(np.int32))
    points = [0, 5, 17, 64, 70]
    expected = opre.segmentation_prefixes(masks, classes, maps, labels, crowd, 3, isthing=[True, False, True],
                                          checkpoints=points)
    actual = pe.segmentation_prefixes(pe.InstanceBatch([_at_offset(m, offset) for m in masks],
                                                       [cuda(c) for c in classes]),
                                      pe.PanopticBatch(cuda(maps), cuda(labels), cuda(crowd)), 3,
                                      isthing=[True, False, True], checkpoints=points)
    compare_snapshots(actual, expected)


def test_large_canvas_histograms_scored_in_place(pe):
    """420 target slots x 65 prefix columns per checkpoint row: too large to stage, scored in place."""
    from panoptic_evaluator_gb300 import synthetic
    images = [synthetic.prefix_one(9, i, side=(70, 70), masks=64, slots=420) for i in range(2)]
    assert len(images[0].target_classes) * (images[0].masks.shape[0] + 1) * 4 > 100 * 1024
    C = 133
    isthing = list(np.arange(C) < 80)
    checkpoints = list(range(8, 65, 8))
    maps = np.stack([i.target for i in images])
    gc = np.stack([i.target_classes for i in images])
    crowd = np.stack([i.crowd for i in images])
    expected = opre.segmentation_prefixes([i.masks for i in images], [i.classes for i in images], maps, gc, crowd, C,
                                          isthing=isthing, checkpoints=checkpoints)
    actual = pe.segmentation_prefixes(pe.InstanceBatch([cuda(i.masks) for i in images],
                                                       [cuda(i.classes) for i in images]),
                                      pe.PanopticBatch(cuda(maps), cuda(gc), cuda(crowd)), C, isthing=isthing,
                                      checkpoints=checkpoints)
    compare_snapshots(actual, expected)
