"""Pin the CPU oracle to the reference: replay the golden inputs and compare.

Integers must match exactly; FP64 values within 1e-12 (NaN == NaN).
"""

import numpy as np
import pytest

from golden_io import load, scalar
from oracle import combined as ocomb
from oracle import instance as oinst
from oracle import panoptic as opan
from oracle import prefix as opre

RTOL = ATOL = 1e-12


def assert_same(actual, expected, path="result"):
    if isinstance(expected, dict):
        assert set(actual) >= set(expected), (path, set(expected) - set(actual))
        for key in expected:
            assert_same(actual[key], expected[key], f"{path}/{key}")
    elif isinstance(expected, list):
        assert len(actual) == len(expected), path
        for i, (a, e) in enumerate(zip(actual, expected)):
            assert_same(a, e, f"{path}/{i}")
    else:
        a, e = np.asarray(actual), np.asarray(expected)
        assert a.shape == e.shape, (path, a.shape, e.shape)
        if e.dtype.kind in "iub":
            np.testing.assert_array_equal(a, e, err_msg=path)
        else:
            np.testing.assert_allclose(a, e, rtol=RTOL, atol=ATOL, equal_nan=True, err_msg=path)


def test_panoptic_matches_reference():
    cases, outputs = load("panoptic")
    for case, expected in zip(cases, outputs):
        oracle = opan.PanopticOracle(int(case["C"]), [bool(x) for x in case["isthing"]], bool(case["validate"]))
        oracle.update(case["pred"], case["pc"], case["gt"], case["gc"], case["crowd"])
        assert_same(oracle.compute(), expected)


def test_original_ids_match_reference():
    inputs, expected = load("original_ids")
    cats = (7, 42, 91)
    t, p = inputs["target"], inputs["prediction"]
    gt_compact = opan.pack(inputs["gt"], t["lookup_ids"], t["lookup_slots"])
    pred_compact = opan.pack(inputs["pred"], p["lookup_ids"], p["lookup_slots"])
    np.testing.assert_array_equal(gt_compact, inputs["gt_compact"])
    np.testing.assert_array_equal(pred_compact, inputs["pred_compact"])
    oracle = opan.PanopticOracle(3)
    oracle.update(pred_compact, p["classes"], gt_compact, t["classes"], t["crowd"])
    assert_same(oracle.compute(), expected)
    # from_coco tables rebuilt from segments_info equal the reference's.
    large = 2**40 + 17
    gi = [[{"id": 1234, "category_id": 7, "iscrowd": 1}, {"id": large, "category_id": 7, "iscrowd": 1},
           {"id": 7, "category_id": 42}], [{"id": 99, "category_id": 91}]]
    ids, slots, classes, crowd = opan.from_coco(inputs["gt"], gi, cats)
    np.testing.assert_array_equal(ids, t["lookup_ids"])
    np.testing.assert_array_equal(slots, t["lookup_slots"])
    np.testing.assert_array_equal(classes, t["classes"])
    np.testing.assert_array_equal(crowd, t["crowd"])


def test_reward_matches_reference():
    cases, outputs = load("reward")
    for case, expected in zip(cases, outputs):
        args = (case["pred"], case["pc"], case["gt"], case["gc"], case["crowd"], int(case["C"]))
        assert_same(opan.panoptic_quality(*args, validate_inputs=False), expected["pq"])
        assert_same(opan.panoptic_quality(*args, validate_inputs=False, return_stats=True), expected["stats"])


def test_matcher_matches_reference():
    cases, outputs = load("matcher")
    for case, expected in zip(cases, outputs):
        pairs = case["pairs"]
        union = np.where(case["crowd"][None], case["pa"][:, None], case["pa"][:, None] + case["ga"][None] - pairs)
        ious = pairs.astype(np.float64) / np.maximum(union, 1)
        status, ranks, counts = oinst.match_ious(ious, case["pc"], case["gc"], case["pa"], case["crowd"],
                                                 case["areas"], int(case["C"]))
        assert_same(dict(status=status, ranks=ranks, counts=counts), expected)


def test_instance_matches_reference():
    cases, outputs = load("instance")
    for case, expected in zip(cases, outputs):
        oracle = oinst.InstanceOracle(int(case["C"]))
        for item in case["images"]:
            oracle.update([item["pm"]], [item["pc"]], [item["scores"]], [item["gm"]], [item["gc"]],
                          [item["crowd"]], [item["areas"]])
        assert_same(oracle.compute(), expected)


def test_combined_matches_reference():
    inputs, expected = load("combined")
    oracle = ocomb.SegmentationOracle(3, [True, True, False])
    for areas in (None, inputs["areas"]):
        oracle.update(inputs["pred_maps"], inputs["classes"], inputs["masks"], inputs["labels"],
                      inputs["scores"], inputs["maps"], inputs["classes"], inputs["crowd"], areas)
    assert_same(oracle.compute(), expected)


def test_prefix_matches_reference():
    cases, outputs = load("prefix")
    for case, expected in zip(cases, outputs):
        checkpoints = None if case["checkpoints"] is None else [int(k) for k in case["checkpoints"]]
        result = opre.segmentation_prefixes(
            [case["masks"]], [case["classes"]], case["maps"], case["labels"], case["crowd"], 3,
            isthing=[True, False, True], checkpoints=checkpoints,
            iou_thresholds=tuple(case["thresholds"].tolist()))
        assert len(result[0]) == len(expected[0])
        for got, want in zip(result[0], expected[0]):
            assert got["prefix"] == scalar(want["prefix"])
            assert_same(got, {k: v for k, v in want.items() if k != "prefix"})


def test_known_answers():
    """Literal known answers from the reference tests (test_evaluator.py:69-101, test_rewards.py:46-48)."""
    o = opan.PanopticOracle(3, [True, False, True])
    o.update(np.array([[[1, 1, 0]]], np.int32), [[-1, 0]], np.array([[[1, 1, 1]]], np.int32), [[-1, 0]])
    r = o.compute()
    assert r["tp"].sum() == 1 and abs(r["iou_sum"].sum() - 2 / 3) < 1e-15
    o = opan.PanopticOracle(3, [True, False, True])
    o.update(np.array([[[1, 0, 1, 2]]], np.int32), [[-1, 0, 1]], np.array([[[1, 1, 2, 2]]], np.int32),
             [[-1, 0, 1]])
    r = o.compute()
    np.testing.assert_array_equal(r["confusion"], [[1, 0, 0, 1], [1, 1, 0, 0], [0, 0, 0, 0]])
    assert abs(r["miou"] - (1 / 3 + 1 / 2) / 2) < 1e-15
    with pytest.raises(ValueError):
        opan.validate(np.array([[[1]]], np.int32), np.array([[-1, -1]], np.int32), None, 3)


def test_rgb_decode_inverts_the_png_encoding():
    """COCO panoptic PNG pixels: id = R + 256 G + 65536 B (README.md:68; encoding of test_evaluator.py:39)."""
    rng = np.random.default_rng(5)
    ids = rng.integers(0, 2**24, (2, 7, 9))
    ids[0, 0, :3] = [0, 2**24 - 1, 65536]
    rgb = opan.encode_rgb(ids)
    assert rgb.dtype == np.uint8 and rgb.shape == (2, 7, 9, 3)
    np.testing.assert_array_equal(opan.decode_rgb(rgb), ids)
    assert tuple(rgb[0, 0, 2]) == (0, 0, 1)
