"""GPU parity of InstanceEvaluator and the instance drop-in ops (reference tests/test_instance.py).

Flags, ranks and counts are bit-exact; precision/recall/summaries within 1e-12.
"""

import numpy as np
import pytest
import torch

from golden_io import load
from helpers import assert_tree, cuda
from oracle import instance as oinst

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pe():
    import panoptic_evaluator_gb300 as pe
    return pe


def batch(pe, *, scores=None, crowd=None):
    masks = torch.zeros((2, 16, 16), dtype=torch.bool, device="cuda")
    masks[0, :10, :10] = True
    masks[1, 5:15, 5:15] = True
    return pe.InstanceBatch([masks], [torch.zeros(2, dtype=torch.int64, device="cuda")],
                            scores=[torch.tensor(scores, device="cuda")] if scores is not None else None,
                            crowd=[torch.tensor(crowd, device="cuda")] if crowd is not None else None)


def test_golden_matcher_cases():
    from panoptic_evaluator_gb300 import _cuda_evaluator as ce
    cases, outputs = load("matcher")
    for case, expected in zip(cases, outputs):
        flags, ranks, counts = ce.instance_match_histogram(
            cuda(case["pairs"]), cuda(case["pc"]), cuda(case["gc"]), cuda(case["pa"]), cuda(case["ga"]),
            cuda(case["crowd"]), cuda(case["areas"]), int(case["C"]))
        np.testing.assert_array_equal(flags.cpu().numpy(), expected["status"])
        np.testing.assert_array_equal(ranks.cpu().numpy(), expected["ranks"])
        np.testing.assert_array_equal(counts.cpu().numpy(), expected["counts"])


def test_golden_instance_cases(pe):
    cases, outputs = load("instance")
    for case, expected in zip(cases, outputs):
        ev = pe.InstanceEvaluator(int(case["C"]))
        for item in case["images"]:
            ev.update(pe.InstanceBatch([cuda(item["pm"])], [cuda(item["pc"])], [cuda(item["scores"])]),
                      pe.InstanceBatch([cuda(item["gm"])], [cuda(item["gc"])], crowd=[cuda(item["crowd"])],
                                       areas=[cuda(item["areas"])]))
        assert_tree(ev.compute(), expected)


def test_golden_instance_cases_one_batch(pe):
    """The same images in one update give the same result as one update per image."""
    cases, outputs = load("instance")
    for case, expected in zip(cases, outputs):
        items = case["images"]
        ev = pe.InstanceEvaluator(int(case["C"]))
        ev.update(pe.InstanceBatch([cuda(i["pm"]) for i in items], [cuda(i["pc"]) for i in items],
                                   [cuda(i["scores"]) for i in items]),
                  pe.InstanceBatch([cuda(i["gm"]) for i in items], [cuda(i["gc"]) for i in items],
                                   crowd=[cuda(i["crowd"]) for i in items], areas=[cuda(i["areas"]) for i in items]))
        assert_tree(ev.compute(), expected)


def test_overlapping_perfect_masks_and_reset(pe):
    ev = pe.InstanceEvaluator(2)
    ev.update(batch(pe, scores=[0.9, 0.8]), batch(pe))
    result = ev.compute()
    assert abs(result["ap"].item() - 1.0) < 1e-12
    assert result["precision"].shape == (10, 101, 2, 4, 3)
    assert (result["precision"][:, :, 1] == -1).all()
    ev.reset()
    assert ev.compute()["ap"].item() == -1.0
    assert abs(result["ap"].item() - 1.0) < 1e-12


def test_missing_predictions_and_crowd(pe):
    empty = pe.InstanceBatch([torch.empty((0, 16, 16), dtype=torch.bool, device="cuda")],
                             [torch.empty(0, dtype=torch.int64, device="cuda")], [torch.empty(0, device="cuda")])
    ev = pe.InstanceEvaluator(1)
    ev.update(empty, batch(pe))
    assert ev.compute()["ap"].item() == 0.0
    ev = pe.InstanceEvaluator(1)
    ev.update(batch(pe, scores=[0.9, 0.8]), batch(pe, crowd=[True, False]))
    ev.update(batch(pe, scores=[0.9, 0.8]), batch(pe))
    assert abs(ev.compute()["ap"].item() - 1.0) < 1e-12


def test_invalid_update_is_atomic(pe):
    ev = pe.InstanceEvaluator(1)
    with pytest.raises(ValueError):
        ev.update(batch(pe), batch(pe))
    assert ev.compute()["ap"].item() == -1.0
    bad_class = pe.InstanceBatch(batch(pe).masks, [torch.tensor([0, 3], device="cuda")],
                                 [torch.tensor([0.9, 0.8], device="cuda")])
    with pytest.raises(ValueError, match="category"):
        ev.update(bad_class, batch(pe))
    empty_mask = batch(pe, scores=[0.9, 0.8])
    empty_mask.masks[0][1].zero_()
    with pytest.raises(ValueError, match="pixels"):
        ev.update(empty_mask, batch(pe))
    with pytest.raises(ValueError, match="finite"):
        ev.update(batch(pe, scores=[float("nan"), 0.8]), batch(pe))
    assert ev.compute()["ap"].item() == -1.0 and ev.num_records == 0


def test_score_order_known_answers(pe):
    target = batch(pe)
    target = pe.InstanceBatch([target.masks[0][:1]], [target.classes[0][:1]])
    ev = pe.InstanceEvaluator(1)
    ev.update(batch(pe, scores=[0.8, 0.9]), target)
    assert abs(ev.compute()["ap"].item() - 0.5) < 1e-12
    ev.reset()
    ev.update(batch(pe, scores=[0.9, 0.8]), target)
    assert abs(ev.compute()["ap"].item() - 1.0) < 1e-12


def test_max_detections_per_category(pe):
    masks = torch.ones((106, 1, 1), dtype=torch.bool, device="cuda")
    labels = torch.zeros(106, dtype=torch.int64, device="cuda")
    labels[-1] = 1
    ev = pe.InstanceEvaluator(2)
    ev.update(pe.InstanceBatch([masks], [labels], [torch.ones(106, device="cuda")]), pe.InstanceBatch([masks], [labels]))
    r = ev.compute()
    for key, k in (("ar1", 1), ("ar10", 10), ("ar100", 100)):
        assert abs(r[key].item() - (k / 105 + 1) / 2) < 1e-12


def test_exact_threshold_and_empty_target(pe):
    pm = torch.tensor([[[True, False]]], device="cuda")
    gm = torch.tensor([[[True, True]]], device="cuda")
    label = torch.tensor([0], device="cuda")
    pred = pe.InstanceBatch([pm], [label], [torch.tensor([0.9], device="cuda")])
    ev = pe.InstanceEvaluator(1)
    ev.update(pred, pe.InstanceBatch([gm], [label]))
    r = ev.compute()
    assert abs(r["ap50"].item() - 1.0) < 1e-12 and abs(r["ap"].item() - 0.1) < 1e-12
    ev.reset()
    ev.update(pred, pe.InstanceBatch([gm[:0]], [label[:0]]))
    assert ev.compute()["ap"].item() == -1.0
    ev.reset()
    ev.update(pe.InstanceBatch([pm[:0]], [label[:0]], [torch.empty(0, device="cuda")]), pe.InstanceBatch([gm], [label]))
    assert ev.compute()["ap"].item() == 0.0


def test_nondefault_stream_snapshots(pe):
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        prediction = batch(pe, scores=[0.9, 0.8])
        target = batch(pe)
        ev = pe.InstanceEvaluator(1, validate=False)
        ev.update(prediction, target)
        prediction.masks[0].zero_()
        prediction.scores[0].zero_()
        result = ev.compute()
        ev.reset()
    stream.synchronize()
    assert abs(result["ap"].item() - 1.0) < 1e-12


def test_drop_in_update_and_compute_ops():
    """instance_update / instance_compute / instance_histogram against the oracle."""
    from panoptic_evaluator_gb300 import _cuda_evaluator as ce
    g = np.random.default_rng(5)
    for D, G, C, h, w in ((9, 6, 3, 24, 37), (40, 12, 2, 17, 19), (0, 5, 2, 8, 8), (7, 0, 2, 8, 8)):
        gm = g.random((G, h, w)) > 0.6
        pm = g.random((D, h, w)) > 0.6
        pc = g.integers(0, C, D).astype(np.int32)
        gc = g.integers(0, C, G).astype(np.int32)
        crowd = g.random(G) < 0.3
        pa = pm.reshape(D, h * w).sum(1).astype(np.float64)
        ga = gm.reshape(G, h * w).sum(1).astype(np.float64)
        areas = g.choice([100.0, 1024.0, 1025.0, 9216.0, 9217.0], G)
        ious = oinst.mask_ious(pm, gm, pa, ga, crowd)
        status, ranks, counts = oinst.match_ious(ious, pc, gc, pa, crowd, areas, C)
        flags, r2, c2 = ce.instance_update(cuda(pm), cuda(gm), cuda(pc), cuda(gc), cuda(pa), cuda(ga), cuda(crowd),
                                           cuda(areas), C)
        np.testing.assert_array_equal(flags.cpu().numpy(), status)
        np.testing.assert_array_equal(r2.cpu().numpy(), ranks)
        np.testing.assert_array_equal(c2.cpu().numpy(), counts)
        order = oinst.score_order(g.random(D))
        precision, recall = ce.instance_compute(cuda(pc[order]), cuda(ranks[order]),
                                                cuda(np.ascontiguousarray(status[:, order])), cuda(counts))
        p_ref, r_ref = oinst.accumulate(pc[order], ranks[order], status[:, order], counts)
        assert_tree([precision, recall], [p_ref, r_ref])
        if D:
            target = g.integers(0, 5, (h, w)).astype(np.int32)
            det_order = g.permutation(D).astype(np.int64)
            pairs = ce.instance_histogram(cuda(pm), cuda(target), cuda(det_order), 5)
            from oracle.combined import detection_histogram
            np.testing.assert_array_equal(pairs.cpu().numpy(), detection_histogram(pm, det_order, target, 5))


def test_config_shaped_instance_batch(pe):
    from panoptic_evaluator_gb300 import synthetic
    images = synthetic.instance_batch(seed=9, images=3, side=(96, 128), gt_range=(1, 20), preds=40)
    C = synthetic.COCO_THINGS
    oracle = oinst.InstanceOracle(C)
    oracle.update([i.pred_masks for i in images], [i.pred_classes for i in images], [i.scores for i in images],
                  [i.gt_masks for i in images], [i.gt_classes for i in images], [i.crowd for i in images])
    ev = pe.InstanceEvaluator(C)
    ev.update(pe.InstanceBatch([cuda(i.pred_masks) for i in images], [cuda(i.pred_classes) for i in images],
                               [cuda(i.scores) for i in images]),
              pe.InstanceBatch([cuda(i.gt_masks) for i in images], [cuda(i.gt_classes) for i in images],
                               crowd=[cuda(i.crowd) for i in images]))
    assert_tree(ev.compute(), oracle.compute())


@pytest.mark.parametrize("sizes", [(300, 700, 1500, 0, 1), (512, 513, 1024, 1025, 40)])
def test_accumulation_of_small_large_and_workspace_classes(sizes):
    """Classes of up to 512 records, 513-1024 records and more than 1024 (sorted in the workspace).

    Records with random ranks, scores (with ties) and chain flags go through the
    accumulation kernel and the oracle's accumulate on the same records in
    global score order; precision and recall agree within 1e-12.
    """
    from types import SimpleNamespace

    from panoptic_evaluator_gb300._batch import Scratch
    from panoptic_evaluator_gb300.instance import accumulate_records
    rng = np.random.default_rng(sum(sizes))
    C = len(sizes)
    classes = np.concatenate([np.full(k, c, np.int32) for c, k in enumerate(sizes)])
    rng.shuffle(classes)
    n = classes.size
    ranks = rng.integers(0, 101, n).astype(np.int32)
    scores = np.round(rng.random(n), 2)  # many ties
    flags = rng.integers(-1, 2, (n, 40)).astype(np.int8)
    counts = rng.integers(0, 400, (C, 4)).astype(np.int64)
    counts[min(3, C - 1)] = 0  # a class without positives
    dev = torch.device("cuda")
    store = SimpleNamespace(n=n, classes=torch.from_numpy(classes).to(dev), ranks=torch.from_numpy(ranks).to(dev),
                            flags=torch.from_numpy(flags).to(dev), scores=torch.from_numpy(scores).to(dev))
    got = accumulate_records(store, torch.from_numpy(counts).to(dev), C, Scratch(dev))
    order = oinst.score_order(scores)
    precision, recall = oinst.accumulate(classes[order], ranks[order], flags.T[:, order], counts)
    np.testing.assert_allclose(got["precision"].cpu().numpy(), precision, rtol=0, atol=1e-12)
    np.testing.assert_allclose(got["recall"].cpu().numpy(), recall, rtol=0, atol=1e-12)


def test_metadata_gather_matches_the_concatenation_path(pe):
    """Per-image classes / scores / crowd / areas of mixed widths gathered on the device equal torch's path.

    Image 0 has int32 classes, float64 scores and float32 areas, image 1 int64 /
    float32 / float64; the same batch with float16 scores (not gathered) takes the
    concatenation path, and every result is the same.
    """
    from panoptic_evaluator_gb300 import instance, synthetic
    images = synthetic.instance_batch(seed=31, images=2, side=(48, 64), gt_range=(2, 12), preds=20)
    dtypes = [(torch.int32, torch.float64, torch.float32), (torch.int64, torch.float32, torch.float64)]

    def batch(score_dtype=None):
        pred = pe.InstanceBatch([cuda(i.pred_masks) for i in images],
                                [cuda(i.pred_classes).to(c) for i, (c, _, _) in zip(images, dtypes)],
                                [cuda(i.scores).to(score_dtype or s) for i, (_, s, _) in zip(images, dtypes)])
        target = pe.InstanceBatch([cuda(i.gt_masks) for i in images],
                                  [cuda(i.gt_classes).to(c) for i, (c, _, _) in zip(images, dtypes)],
                                  crowd=[cuda(i.crowd) for i in images],
                                  areas=[cuda(i.gt_masks.sum((1, 2)).astype(np.float64)).to(a) + 0.5
                                         for i, (_, _, a) in zip(images, dtypes)])
        return pred, target

    pred, target = batch()
    assert instance.gather_rows(pred, target, 2) is not None
    half = batch(torch.float16)
    assert instance.gather_rows(*half, 2) is None
    results = []
    for p, t in ((pred, target), (half[0], target)):
        ev = pe.InstanceEvaluator(synthetic.COCO_THINGS)
        # float16 scores differ from the others' values: compare each path with its own torch-path run below
        ev.update(p, t)
        results.append(ev.compute())
    saved = instance.gather_rows
    try:
        instance.gather_rows = lambda *a: None  # force the concatenation path
        for k, (p, t) in enumerate(((pred, target), (half[0], target))):
            ev = pe.InstanceEvaluator(synthetic.COCO_THINGS)
            ev.update(p, t)
            assert_tree(ev.compute(), results[k])
    finally:
        instance.gather_rows = saved
