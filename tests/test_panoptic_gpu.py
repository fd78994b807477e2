"""GPU parity of PanopticEvaluator / panoptic_quality against the oracle and the golden vectors.

Mirrors the reference's tests/test_evaluator.py and tests/test_rewards.py.
Integers are bit-exact; FP64 within 1e-12.
"""

import numpy as np
import pytest
import torch

from golden_io import load
from helpers import assert_tree, cuda
from oracle import panoptic as opan

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pe():
    import panoptic_evaluator_gb300 as pe
    return pe


def evaluate(pe, gt, pred, gi, pi, categories=(7, 42, 91), isthing=(True, False, True), validate=True):
    ev = pe.PanopticEvaluator(3, isthing=list(isthing), validate=validate)
    t = pe.PanopticBatch.from_coco(torch.tensor(gt, dtype=torch.int64, device="cuda"), gi, categories)
    p = pe.PanopticBatch.from_coco(torch.tensor(pred, dtype=torch.int64, device="cuda"), pi, categories)
    ev.update(p, t)
    return ev


def test_golden_panoptic_cases(pe):
    cases, outputs = load("panoptic")
    for case, expected in zip(cases, outputs):
        ev = pe.PanopticEvaluator(int(case["C"]), isthing=[bool(x) for x in case["isthing"]],
                                  validate=bool(case["validate"]))
        crowd = None if case["crowd"] is None else cuda(case["crowd"])
        ev.update(pe.PanopticBatch(cuda(case["pred"]), cuda(case["pc"])),
                  pe.PanopticBatch(cuda(case["gt"]), cuda(case["gc"]), crowd))
        assert_tree(ev.compute(), expected)


def test_perfect_and_reset(pe):
    maps = [[[0, 1, 1, 2]]]
    info = [[{"id": 1, "category_id": 7}, {"id": 2, "category_id": 42}]]
    ev = evaluate(pe, maps, maps, info, info)
    r = ev.compute()
    assert r["All"]["pq"].item() == 1 and r["Things"]["n"].item() == 1 and r["Stuff"]["pq"].item() == 1
    assert torch.isnan(r["per_class"]["iou"][2]) and r["miou"].item() == 1
    ev.reset()
    assert ev.compute()["All"]["pq"].item() == 0 and ev.compute()["miou"].item() == 0


def test_strict_half_void_union_crowd(pe):
    gi = [[{"id": 1, "category_id": 7}]]
    pi = [[{"id": 9, "category_id": 7}]]
    r = evaluate(pe, [[[1, 1, 1, 1]]], [[[9, 9, 0, 0]]], gi, pi).compute()
    assert (r["tp"].sum().item(), r["fp"].sum().item(), r["fn"].sum().item()) == (0, 1, 1)
    assert r["miou"].item() == .5
    r = evaluate(pe, [[[1, 1, 1]]], [[[9, 9, 0]]], gi, pi).compute()
    assert r["tp"].sum().item() == 1 and abs(r["iou_sum"].sum().item() - 2 / 3) < 1e-15
    assert evaluate(pe, [[[1, 0, 0, 0]]], [[[9, 9, 9, 9]]], gi, pi).compute()["All"]["pq"].item() == 1
    gc = [[{"id": 1, "category_id": 7, "iscrowd": 1}]]
    r = evaluate(pe, [[[1, 1, 0]]], [[[9, 9, 9]]], gc, pi).compute()
    assert r["fp"].sum().item() == 0 and r["fn"].sum().item() == 0
    r = evaluate(pe, [[[1, 1, 1, 1]]], [[[9, 9, 9, 9]]], gc, [[{"id": 9, "category_id": 42}]]).compute()
    assert r["fp"][1].item() == 1
    r = evaluate(pe, [[[0, 0, 1, 1]]], [[[9, 9, 9, 9]]], [[{"id": 1, "category_id": 42}]], pi).compute()
    assert r["fp"][0].item() == 1


def test_semantic_confusion_known_answer(pe):
    r = evaluate(pe, [[[1, 1, 2, 2]]], [[[9, 0, 9, 10]]],
                 [[{"id": 1, "category_id": 7}, {"id": 2, "category_id": 42}]],
                 [[{"id": 9, "category_id": 7}, {"id": 10, "category_id": 42}]]).compute()
    assert r["confusion"].cpu().tolist() == [[1, 0, 0, 1], [1, 1, 0, 0], [0, 0, 0, 0]]
    assert abs(r["miou"].item() - (1 / 3 + 1 / 2) / 2) < 1e-15


def test_original_ids_all_paths_match_golden(pe):
    inputs, expected = load("original_ids")
    t, p = inputs["target"], inputs["prediction"]

    def batch(maps, tables, dtype):
        return pe.PanopticBatch(cuda(maps, dtype), cuda(tables["classes"]), cuda(tables["crowd"]),
                                cuda(tables["lookup_ids"]), cuda(tables["lookup_slots"]))
    for gt_dtype, pred_dtype in ((torch.int64, torch.int64), (torch.int64, torch.int32), (torch.int32, torch.int64)):
        target = batch(inputs["gt"], t, gt_dtype) if gt_dtype == torch.int64 else None
        if target is None:
            continue
        prediction = batch(inputs["pred"], p, pred_dtype)
        np.testing.assert_array_equal(target.compact().segment_map.cpu(), inputs["gt_compact"])
        np.testing.assert_array_equal(prediction.compact().segment_map.cpu(), inputs["pred_compact"])
        for validate in (True, False):
            for ct, cp in ((False, False), (True, False), (False, True)):
                ev = pe.PanopticEvaluator(3, validate=validate)
                ev.update(prediction.compact() if cp else prediction, target.compact() if ct else target)
                assert_tree(ev.compute(), expected)


def test_original_ids_across_image_boundaries(pe):
    maps = np.array([[[11, 22, 11, 0, 22, 11, 22, 11, 22, 11, 22, 11, 22, 11, 22, 11, 22]]] * 3, np.int64)
    info = [[{"id": 11, "category_id": 7}, {"id": 22, "category_id": 42}],
            [{"id": 22, "category_id": 7}, {"id": 11, "category_id": 42}],
            [{"id": 11, "category_id": 42}, {"id": 22, "category_id": 7}]]
    ids, slots, classes, crowd = opan.from_coco(maps, info, (7, 42))
    compact = opan.pack(maps, ids, slots)
    oracle = opan.PanopticOracle(2)
    oracle.update(compact, classes, compact, classes, crowd)
    original = pe.PanopticBatch.from_coco(torch.tensor(maps, device="cuda"), info, (7, 42), compact=False)
    np.testing.assert_array_equal(original.compact().segment_map.cpu(), compact)
    for validate in (False, True):
        ev = pe.PanopticEvaluator(2, validate=validate)
        ev.update(original, original)
        assert_tree(ev.compute(), oracle.compute())


def test_validation_preserves_previous_totals(pe):
    maps = torch.tensor([[[1, 1]]], dtype=torch.int32, device="cuda")
    classes = torch.tensor([[-1, 0]], dtype=torch.int32, device="cuda")
    good = pe.PanopticBatch(maps, classes)
    ev = pe.PanopticEvaluator(3)
    ev.update(good, good)
    before = ev.compute()
    unknown = pe.PanopticBatch.from_coco(torch.tensor([[[7, 8]]], dtype=torch.int64, device="cuda"),
                                         [[{"id": 7, "category_id": 7}]], (7, 42, 91), compact=False)
    bad_batches = [pe.PanopticBatch(maps + 3, classes),
                   pe.PanopticBatch(maps, torch.tensor([[-1, 4]], dtype=torch.int32, device="cuda")),
                   pe.PanopticBatch(maps, torch.tensor([[-1, -1]], dtype=torch.int32, device="cuda")),
                   pe.PanopticBatch(maps, torch.tensor([[-1, 0, 1]], dtype=torch.int32, device="cuda")),
                   pe.PanopticBatch(maps, classes, torch.tensor([[True, False]], device="cuda")),
                   unknown]
    for index, bad in enumerate(bad_batches):
        with pytest.raises(ValueError):
            ev.update(good, bad)
        if index != 4:
            with pytest.raises(ValueError):
                ev.update(bad, good)
        assert_tree(ev.compute(), before, exact_float=True)


def test_empty_and_noncontiguous(pe):
    for shape in ((0, 3, 4), (2, 0, 4)):
        batch = pe.PanopticBatch(torch.empty(shape, dtype=torch.int32, device="cuda"),
                                 torch.full((shape[0], 1), -1, dtype=torch.int32, device="cuda"))
        ev = pe.PanopticEvaluator(3)
        ev.update(batch, batch)
        assert ev.compute()["confusion"].sum().item() == 0
    empty = pe.PanopticBatch.from_coco(torch.zeros((1, 1, 2), dtype=torch.int64, device="cuda"), [[]], (7, 42, 91))
    ev = pe.PanopticEvaluator(3)
    ev.update(empty, empty)
    assert ev.compute()["All"]["n"].item() == 0
    prediction = pe.PanopticBatch.from_coco(torch.ones((1, 1, 2), dtype=torch.int64, device="cuda"),
                                            [[{"id": 1, "category_id": 7}]], (7, 42, 91))
    ev.update(prediction, empty)  # predictions entirely on void are ignored
    assert ev.compute()["fp"].sum().item() == 0
    ev.update(empty, prediction)
    assert ev.compute()["fn"][0].item() == 1 and ev.compute()["miou"].item() == 0
    maps = torch.ones((2, 4, 6), device="cuda", dtype=torch.int32)[:, ::2, ::2]
    labels = torch.tensor([[-1, -1, 0, -1]], device="cuda", dtype=torch.int32)[:, ::2].expand(2, -1)
    ev.reset()
    ev.update(pe.PanopticBatch(maps, labels), pe.PanopticBatch(maps, labels))
    assert ev.compute()["All"]["pq"].item() == 1


@pytest.mark.parametrize("G,P", [(1, 1), (2, 3), (65, 97), (137, 193), (257, 513), (1025, 769)])
def test_varied_capacities_and_snapshots(pe, G, P):
    """Shared-memory and global-atomic histograms, P >= 128 columns, crowd and void."""
    g = np.random.default_rng(857 + G)
    gt = g.integers(0, G, (3, 31, 47)).astype(np.int32)
    pred = g.integers(0, P, gt.shape).astype(np.int32)
    gc = g.integers(0, 5, (3, G)).astype(np.int32)
    pc = g.integers(0, 5, (3, P)).astype(np.int32)
    gc[:, 0] = pc[:, 0] = -1
    crowd = g.random((3, G)) < .25
    crowd[:, 0] = False
    if G == 65:
        pred = gt.copy()
        pc[:, :G] = gc
        pc[:, G:] = -1
        pred[:, ::5, :] = 0
    oracle = opan.PanopticOracle(5, validate=False)
    oracle.update(pred, pc, gt, gc, crowd)
    ev = pe.PanopticEvaluator(5, validate=False)
    ev.update(pe.PanopticBatch(cuda(pred), cuda(pc)), pe.PanopticBatch(cuda(gt), cuda(gc), cuda(crowd)))
    snapshot = ev.compute()
    assert_tree(snapshot, oracle.compute())
    saved = {k: snapshot[k].clone() for k in ("tp", "fp", "fn", "iou_sum", "confusion")}
    pointers = tuple(t.data_ptr() for t in ev._scratch)
    ev.reset()
    ev.update(pe.PanopticBatch(cuda(pred), cuda(pc)), pe.PanopticBatch(cuda(gt), cuda(gc), cuda(crowd)))
    assert tuple(t.data_ptr() for t in ev._scratch) == pointers
    for key in saved:
        torch.testing.assert_close(snapshot[key], saved[key], rtol=0, atol=0)


def test_cooperative_rows_with_validation(pe):
    maps = np.arange(1, 130, dtype=np.int32).reshape(1, 3, 43)
    gc = np.full((1, 137), -1, np.int32)
    pc = np.full((1, 193), -1, np.int32)
    gc[:, 1:130] = pc[:, 1:130] = np.arange(129) % 3
    oracle = opan.PanopticOracle(3)
    oracle.update(maps, pc, maps, gc)
    for validate in (False, True):
        ev = pe.PanopticEvaluator(3, validate=validate)
        ev.update(pe.PanopticBatch(cuda(maps), cuda(pc)), pe.PanopticBatch(cuda(maps), cuda(gc)))
        assert_tree(ev.compute(), oracle.compute())


def test_graph_capture_reuses_scratch(pe):
    maps = torch.tensor([[[1, 1, 2, 2]]], dtype=torch.int32, device="cuda")
    classes = torch.tensor([[-1, 0, 1]], dtype=torch.int32, device="cuda")
    compact = pe.PanopticBatch(maps, classes)
    original = pe.PanopticBatch.from_coco(maps.long() * 100003 + 2**40,
                                          [[{"id": 100003 + 2**40, "category_id": 7},
                                            {"id": 200006 + 2**40, "category_id": 42}]], (7, 42, 91), compact=False)
    for item in (compact, original):
        ev = pe.PanopticEvaluator(3, validate=False)
        stream = torch.cuda.Stream()
        stream.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(stream):
            ev.update(item, item)
        torch.cuda.current_stream().wait_stream(stream)
        ev.reset()
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            ev.update(item, item)
        graph.replay()
        graph.replay()
        assert ev.compute()["tp"].cpu().tolist() == [2, 2, 0]


def test_nondefault_stream_exact(pe):
    stream = torch.cuda.Stream()
    g = torch.Generator(device="cuda").manual_seed(5)
    with torch.cuda.stream(stream):
        gt = torch.randint(0, 17, (4, 128, 129), device="cuda", dtype=torch.int32, generator=g)
        pred = torch.randint(0, 21, gt.shape, device="cuda", dtype=torch.int32, generator=g)
        gc = torch.arange(17, device="cuda", dtype=torch.int32)[None].expand(4, -1).clone() % 3
        pc = torch.arange(21, device="cuda", dtype=torch.int32)[None].expand(4, -1).clone() % 3
        gc[:, 0] = pc[:, 0] = -1
        crowd = torch.zeros_like(gc, dtype=torch.bool)
        crowd[:, 3] = True
        ev = pe.PanopticEvaluator(3)
        ev.update(pe.PanopticBatch(pred, pc), pe.PanopticBatch(gt, gc, crowd))
        result = ev.compute()
    stream.synchronize()
    oracle = opan.PanopticOracle(3)
    oracle.update(pred.cpu().numpy(), pc.cpu().numpy(), gt.cpu().numpy(), gc.cpu().numpy(), crowd.cpu().numpy())
    expected = oracle.compute()
    for key in ("confusion", "tp", "fp", "fn"):
        np.testing.assert_array_equal(result[key].cpu().numpy(), expected[key])
    np.testing.assert_allclose(result["iou_sum"].cpu().numpy(), expected["iou_sum"], rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("workload", ["voronoi", "coco"])
def test_config_shaped_batches(pe, workload):
    from panoptic_evaluator_gb300 import synthetic
    a = synthetic.voronoi_batch(seed=3) if workload == "voronoi" else synthetic.coco_panoptic_batch(seed=4, B=4)
    oracle = opan.PanopticOracle(a.num_classes, a.isthing)
    oracle.update(a.pred, a.pc, a.gt, a.gc, a.crowd)
    for validate in (True, False):
        ev = pe.PanopticEvaluator(a.num_classes, isthing=a.isthing.tolist(), validate=validate)
        ev.update(pe.PanopticBatch(cuda(a.pred), cuda(a.pc)), pe.PanopticBatch(cuda(a.gt), cuda(a.gc), cuda(a.crowd)))
        assert_tree(ev.compute(), oracle.compute())
    stats = pe.panoptic_quality(pe.PanopticBatch(cuda(a.pred), cuda(a.pc)),
                                pe.PanopticBatch(cuda(a.gt), cuda(a.gc), cuda(a.crowd)), a.num_classes,
                                return_stats=True)
    assert_tree(stats, opan.panoptic_quality(a.pred, a.pc, a.gt, a.gc, a.crowd, a.num_classes, return_stats=True))


def test_reward_golden_and_metadata_reuse(pe):
    cases, outputs = load("reward")
    for case, expected in zip(cases, outputs):
        t = pe.PanopticBatch(cuda(case["gt"]), cuda(case["gc"]), cuda(case["crowd"]))
        p = pe.PanopticBatch(cuda(case["pred"]), cuda(case["pc"]))
        assert_tree(pe.panoptic_quality(p, t, int(case["C"]), validate=False), expected["pq"])
        assert_tree(pe.panoptic_quality(p, t, int(case["C"]), validate=False, return_stats=True), expected["stats"])
    case, expected = cases[0], outputs[0]
    gt, pred, gc, pc, crowd = (case[k] for k in ("gt", "pred", "gc", "pc", "crowd"))
    pq = pe.panoptic_quality(pe.PanopticBatch(cuda(pred), cuda(pc)), pe.PanopticBatch(cuda(gt), cuda(gc), cuda(crowd)),
                             4, validate=True)
    assert_tree(pq, expected["pq"])
    ids = [0, 2**40 + 9, 71]
    gi = [[dict(id=ids[s], category_id=int(gc[b, s]), iscrowd=bool(crowd[b, s])) for s in (1, 2) if gc[b, s] >= 0]
          for b in range(8)]
    pi = [[dict(id=ids[s], category_id=int(pc[b, s])) for s in (1, 2)] for b in range(8)]
    original = torch.tensor(ids, device="cuda")
    prepared_gt = pe.PanopticBatch.from_coco(original[cuda(gt).long()], gi, range(4), compact=False)
    prepared_pred = pe.PanopticBatch.from_coco(original[cuda(pred).long()], pi, range(4), compact=False)
    assert_tree(pe.panoptic_quality(prepared_pred, prepared_gt, 4), expected["pq"])
    empty = prepared_pred.with_maps(torch.zeros_like(prepared_pred.segment_map))
    assert_tree(pe.panoptic_quality(empty, prepared_gt, 4), np.zeros(8))


def test_reward_invalid_inputs(pe):
    batch = pe.PanopticBatch(torch.ones((1, 1, 2), device="cuda", dtype=torch.int32),
                             torch.tensor([[-1, 0]], device="cuda", dtype=torch.int32))
    assert pe.panoptic_quality(batch, batch, 1).item() == 1
    with pytest.raises(ValueError):
        pe.panoptic_quality(batch, batch, 1, reduction="mean")
    with pytest.raises(ValueError):
        pe.panoptic_quality(batch.with_maps(torch.full_like(batch.segment_map, 9)), batch, 1)
    with pytest.raises(ValueError):
        pe.PanopticEvaluator(1).update(batch.with_maps(torch.zeros_like(batch.segment_map)), batch)
