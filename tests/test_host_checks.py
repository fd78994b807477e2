"""Structural argument checks of the batched evaluators, run on CPU tensors (no GPU work).

The messages are the reference's (panoptic_evaluator/instance.py:78-126 and
prefix.py:31-60); value checks (finite scores, class ranges, empty masks) run on
the GPU and are covered by the GPU tests.
"""

import pytest
import torch

from panoptic_evaluator_gb300.instance import InstanceBatch, check_instance_batch, gather_rows, shape_table

CPU = torch.device("cpu")


def _batch(n=(3, 2), hw=(4, 5), scores=True, crowd=False, areas=False):
    masks = [torch.zeros((k, *hw), dtype=torch.bool) for k in n]
    classes = [torch.zeros(k, dtype=torch.int64) for k in n]
    return InstanceBatch(masks, classes, [torch.rand(k) for k in n] if scores else None,
                         crowd=[torch.zeros(k, dtype=torch.bool) for k in n] if crowd else None,
                         areas=[torch.ones(k, dtype=torch.float64) for k in n] if areas else None)


def _replace(batch, **fields):
    values = dict(masks=batch.masks, classes=batch.classes, scores=batch.scores, crowd=batch.crowd, areas=batch.areas)
    values.update(fields)
    return InstanceBatch(values.pop("masks"), values.pop("classes"), values.pop("scores"), **values)


def test_valid_batches_return_shapes_and_dtypes():
    pred = _batch()
    shapes, dtypes = check_instance_batch(pred, CPU, prediction=True)
    assert [tuple(s) for s in shapes] == [(3, 4, 5), (2, 4, 5)]
    assert shape_table(shapes).tolist() == [[3, 4, 5], [2, 4, 5]]
    assert set(dtypes) == {"classes", "scores"} and dtypes["scores"] == [torch.float32] * 2
    target = _batch(scores=False, crowd=True, areas=True)
    _, dtypes = check_instance_batch(target, CPU, prediction=False)
    assert set(dtypes) == {"classes", "crowd", "areas"}
    rows = gather_rows(pred, target, 2, (check_instance_batch(pred, CPU, prediction=True)[1], dtypes))
    assert rows is not None and list(rows[:, 5]) == [1 | 4 | 16] * 2  # int64 classes, float64 areas


@pytest.mark.parametrize("case, message", [
    ("field_count", "all fields must contain one tensor per image"),
    ("no_scores", "predictions require scores"),
    ("mask_dims", "masks must be bool N x H x W with positive image dimensions"),
    ("mask_empty_side", "masks must be bool N x H x W with positive image dimensions"),
    ("mask_dtype", "masks must be bool N x H x W with positive image dimensions"),
    ("class_shape", "classes must be int32/int64 N tensors"),
    ("class_dtype", "classes must be int32/int64 N tensors"),
    ("score_shape", "scores must have shape N and share evaluator device"),
    ("score_dtype", "scores must be floating point"),
    ("crowd_dtype", "crowd must be bool"),
    ("area_dtype", "areas must be floating point"),
    ("device", "inputs must share evaluator device"),
])
def test_each_fault_raises_the_reference_message(case, message):
    good = _batch(crowd=True, areas=True)
    device = CPU
    if case == "field_count":
        batch = _replace(good, classes=good.classes[:1])
    elif case == "no_scores":
        batch = _replace(good, scores=None)
    elif case == "mask_dims":
        batch = _replace(good, masks=[good.masks[0], torch.zeros((2, 20), dtype=torch.bool)])
    elif case == "mask_empty_side":
        batch = _replace(good, masks=[good.masks[0], torch.zeros((2, 0, 5), dtype=torch.bool)])
    elif case == "mask_dtype":
        batch = _replace(good, masks=[good.masks[0], good.masks[1].to(torch.uint8)])
    elif case == "class_shape":
        batch = _replace(good, classes=[good.classes[0], torch.zeros(3, dtype=torch.int64)])
    elif case == "class_dtype":
        batch = _replace(good, classes=[good.classes[0], good.classes[1].float()])
    elif case == "score_shape":
        batch = _replace(good, scores=[good.scores[0], torch.rand(5)])
    elif case == "score_dtype":
        batch = _replace(good, scores=[good.scores[0], torch.ones(2, dtype=torch.int32)])
    elif case == "crowd_dtype":
        batch = _replace(good, crowd=[good.crowd[0], torch.zeros(2, dtype=torch.uint8)])
    elif case == "area_dtype":
        batch = _replace(good, areas=[good.areas[0], torch.ones(2, dtype=torch.int64)])
    else:  # masks and classes on another device than the evaluator's (no metadata fields to trip first)
        batch = _replace(good, scores=None, crowd=None, areas=None)
        device = torch.device("meta")
    with pytest.raises(ValueError, match=message):
        check_instance_batch(batch, device, prediction=case != "device")


def test_prefix_argument_checks():
    from panoptic_evaluator_gb300.prefix import _check_arguments, check_prefix_inputs
    assert _check_arguments((0.5, 0.75), (8, 16)) == ((0.5, 0.75), (8, 16))
    for thresholds in ((), (0.0,), (1.5,), (float("nan"),), (True,)):
        with pytest.raises(ValueError, match="iou_thresholds"):
            _check_arguments(thresholds, None)
    for points in ((8, 8), (16, 8), (-1,), (1.0,)):
        with pytest.raises(ValueError, match="checkpoints"):
            _check_arguments((0.5,), points)
    masks = [torch.zeros((3, 4, 5), dtype=torch.bool), torch.zeros((2, 4, 5), dtype=torch.bool)]
    classes = [torch.zeros(3, dtype=torch.int32), torch.zeros(2, dtype=torch.int32)]
    counts = check_prefix_inputs(masks, classes, (2, 4, 5), CPU, (1, 2))
    assert counts.tolist() == [3, 2]
    with pytest.raises(ValueError, match="matching batch and image dimensions"):
        check_prefix_inputs(masks, classes, (2, 4, 6), CPU, None)
    with pytest.raises(ValueError, match="matching batch and image dimensions"):
        check_prefix_inputs(masks[:1], classes[:1], (2, 4, 5), CPU, None)
    with pytest.raises(ValueError, match="all fields must contain one tensor per image"):
        check_prefix_inputs(masks, classes[:1], (2, 4, 5), CPU, None)
    # The instance checks come first, with the reference's messages.
    with pytest.raises(ValueError, match="masks must be bool N x H x W with positive image dimensions"):
        check_prefix_inputs([masks[0], torch.zeros((2, 20), dtype=torch.bool)], classes, (3, 4, 5), CPU, None)
    with pytest.raises(ValueError, match="masks must be bool N x H x W with positive image dimensions"):
        check_prefix_inputs([masks[0], masks[1].to(torch.uint8)], classes, (2, 4, 5), CPU, None)
    with pytest.raises(ValueError, match="classes must be int32/int64 N tensors"):
        check_prefix_inputs(masks, [classes[0], torch.zeros(3, dtype=torch.int32)], (2, 4, 5), CPU, None)
    with pytest.raises(ValueError, match="inputs must share evaluator device"):
        check_prefix_inputs(masks, classes, (2, 4, 5), torch.device("meta"), None)
    with pytest.raises(ValueError, match="checkpoint exceeds prediction count"):
        check_prefix_inputs(masks, classes, (2, 4, 5), CPU, (1, 3))
    assert check_prefix_inputs([], [], (0, 4, 5), CPU, None) is None
