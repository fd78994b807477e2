"""Update autotuner: cache format and bucket keys on the CPU; tuned launches on the GPU."""

import json

import numpy as np
import pytest
import torch


def test_bucket_keys_and_cache_round_trip(tmp_path, monkeypatch):
    from panoptic_evaluator_gb300 import tuning
    assert tuning.bucket(12221, 409600) == (13, 18)
    assert tuning.bucket(1, 1) == (0, 0)
    calls = []
    monkeypatch.setattr(tuning.N, "call", lambda name, *args: calls.append((name, args)) or 0)
    path = tmp_path / "tuning.json"
    tuning.write([{"bins_bucket": 13, "pixels_bucket": 18, "smem": 1, "ctas_per_sm": 2, "score_threads": 256}], path)
    tuning.write([{"bins_bucket": 13, "pixels_bucket": 18, "smem": 0, "ctas_per_sm": 4, "score_threads": 1024},
                  {"bins_bucket": 6, "pixels_bucket": 12, "smem": 1, "ctas_per_sm": 1, "score_threads": 512}], path)
    assert len(json.loads(path.read_text())["update"]) == 2  # one entry per bucket, the newest wins
    assert tuning.load(path) == 2
    assert sorted(calls) == [("pe_tune_update", (1 << 6, 1 << 12, 1, 1, 512)),
                             ("pe_tune_update", (1 << 13, 1 << 18, 0, 4, 1024))]


@pytest.mark.gpu
def test_every_update_choice_counts_the_same():
    import panoptic_evaluator_gb300 as pe
    from panoptic_evaluator_gb300 import tuning
    rng = np.random.default_rng(3)
    B, H, W, G, P, C = 3, 97, 131, 37, 45, 20
    dev = torch.device("cuda")
    gt = torch.from_numpy(tuning._maps(rng, B, H, W, G, 9)).to(dev)
    pr = torch.from_numpy(tuning._maps(rng, B, H, W, P, 5)).to(dev)
    gc = torch.from_numpy(rng.integers(-1, C, (B, G)).astype(np.int32)).to(dev)
    pc = torch.from_numpy(rng.integers(-1, C, (B, P)).astype(np.int32)).to(dev)
    gc[:, 0] = pc[:, 0] = -1
    key = tuning.bucket(G * P, H * W)
    results = []
    try:
        for smem in (1, 0):
            for per_sm in tuning.CTAS_PER_SM:
                for threads in tuning.SCORE_THREADS:
                    tuning.register(*key, smem, per_sm, threads)
                    assert tuning.choice(G * P, H * W) == (smem, per_sm, threads)
                    ev = pe.PanopticEvaluator(C, device=dev, validate=False)
                    ev.update(pe.PanopticBatch(pr, pc), pe.PanopticBatch(gt, gc))
                    results.append({k: v.clone() for k, v in ev.state_dict().items()})
                    rewards = pe.panoptic_quality(pe.PanopticBatch(pr, pc), pe.PanopticBatch(gt, gc), C,
                                                  validate=False)
                    results[-1]["reward"] = rewards.clone()
    finally:
        tuning.forget(*key)
    for r in results[1:]:
        for k, v in r.items():
            assert torch.equal(v, results[0][k]), k


@pytest.mark.gpu
def test_tuner_keeps_the_fastest_candidate():
    from panoptic_evaluator_gb300 import tuning
    out = tuning.tune_update(33, 41, 160, 200, images=4, repeats=2)
    assert len(out["candidates"]) == 8 and out["ms"] == min(c["ms"] for c in out["candidates"])
    assert tuning.choice(33 * 41, 160 * 200) == (out["smem"], out["ctas_per_sm"], out["score_threads"])
    tuning.forget(*tuning.bucket(33 * 41, 160 * 200))


def test_pass_cache_shares_the_file_with_update_entries(tmp_path, monkeypatch):
    from panoptic_evaluator_gb300 import tuning
    calls = []
    monkeypatch.setattr(tuning.N, "call", lambda name, *args: calls.append((name, args)) or 0)
    path = tmp_path / "tuning.json"
    tuning.write([{"bins_bucket": 13, "pixels_bucket": 18, "smem": 1, "ctas_per_sm": 2, "score_threads": 256}], path)
    tuning.write_pass([{"chunks_bucket": 14, "grab": 2, "ctas_per_sm": 1}], path)
    tuning.write_pass([{"chunks_bucket": 14, "grab": 4, "ctas_per_sm": 2},
                       {"chunks_bucket": 9, "grab": 1, "ctas_per_sm": 2}], path)
    tuning.write([{"bins_bucket": 6, "pixels_bucket": 12, "smem": 0, "ctas_per_sm": 1, "score_threads": 512}], path)
    data = json.loads(path.read_text())
    assert len(data["update"]) == 2 and len(data["pass"]) == 2  # neither writer drops the other's entries
    assert tuning.load(path) == 4
    assert sorted(c for c in calls if c[0] == "pe_tune_pass") == [("pe_tune_pass", (1 << 9, 1, 2)),
                                                                  ("pe_tune_pass", (1 << 14, 4, 2))]


@pytest.mark.gpu
def test_every_pass_choice_counts_the_same():
    """Each (chunks per grab, CTAs per SM) choice of the batched pass gives the oracle's results."""
    import panoptic_evaluator_gb300 as pe
    from helpers import assert_tree
    from oracle import combined as ocomb
    from panoptic_evaluator_gb300 import synthetic, tuning
    from panoptic_evaluator_gb300.ragged import SegmentationImages
    images = synthetic.segmentation_batch(seed=17, images=12, side=(100, 400), slots=(5, 60), dets=(0, 40))
    C = 133
    isthing = list(np.arange(C) < 80)
    oracle = ocomb.SegmentationOracle(C, isthing)
    for i in images:
        oracle.update(i.pred[None], i.pred_classes[None], [i.det_masks], [i.det_classes], [i.scores], i.target[None],
                      i.target_classes[None], i.crowd[None])
    expected = oracle.compute()
    arena = SegmentationImages([i.target for i in images], [i.target_classes for i in images],
                               [i.crowd for i in images], [i.pred for i in images], [i.pred_classes for i in images],
                               [i.det_masks for i in images], [i.det_classes for i in images],
                               [i.scores for i in images])
    ev = pe.SegmentationEvaluator(C, isthing=isthing)
    chunks = arena.table(ev.instance._scratch).total_chunks
    key = int(np.floor(np.log2(chunks)))
    try:
        for grab in tuning.PASS_GRABS:
            for per_sm in tuning.PASS_CTAS_PER_SM:
                tuning.register_pass(key, grab, per_sm)
                assert tuning.pass_choice(chunks) == (grab, per_sm)
                ev.reset()
                ev.update_images(arena)
                assert_tree(ev.compute(), expected)
        result = tuning.tune_pass(ev, arena, repeats=2)
        assert len(result["candidates"]) == 6 and tuning.pass_choice(chunks) == (result["grab"], result["ctas_per_sm"])
    finally:
        tuning.forget_pass(key)
    assert tuning.pass_choice(chunks) == (1, 2)


def test_contract_bucket_and_cache_round_trip(tmp_path):
    """Buckets are tenths of the mask bytes loaded by TMA; contraction entries share the cache file."""
    from panoptic_evaluator_gb300 import tuning
    from panoptic_evaluator_gb300._batch import CONTRACT_TMA_COST
    dets, gts, pixels = [10, 20, 30], [5, 5, 10], [100, 100, 1000]  # mask bytes 1500, 2500, 40000
    assert tuning.contract_bucket(dets, gts, pixels, [False, False, False]) == 0
    assert tuning.contract_bucket(dets, gts, pixels, [True, True, False]) == 0  # 4000 / 44000
    assert tuning.contract_bucket(dets, gts, pixels, [False, False, True]) == 9  # 40000 / 44000
    assert tuning.contract_bucket(dets, gts, pixels, [True, True, True]) == 10
    assert tuning.contract_bucket([0], [0], [100], [True]) == 0
    path = tmp_path / "tuning.json"
    tuning.write_pass([{"chunks_bucket": 9, "grab": 1, "ctas_per_sm": 2}], path)
    tuning.write_contract([{"tma_bucket": 2, "tma_cost": 0.5}], path)
    tuning.write_contract([{"tma_bucket": 2, "tma_cost": 0.7}, {"tma_bucket": 10, "tma_cost": 1.0}], path)
    data = json.loads(path.read_text())
    assert len(data["pass"]) == 1 and data["contract"] == [{"tma_bucket": 2, "tma_cost": 0.7},
                                                           {"tma_bucket": 10, "tma_cost": 1.0}]
    try:
        for e in tuning.read_contract(path):
            tuning.register_contract(e["tma_bucket"], e["tma_cost"])
        assert tuning.contract_cost(2) == 0.7 and tuning.contract_cost(10) == 1.0
        assert tuning.contract_cost(5) == CONTRACT_TMA_COST
    finally:
        tuning.forget_contract(2)
        tuning.forget_contract(10)
    assert tuning.contract_cost(2) == CONTRACT_TMA_COST


@pytest.mark.gpu
def test_every_contract_split_counts_the_same():
    """Each TMA block weight of the contraction's CTA split gives the oracle's instance results."""
    import torch

    import panoptic_evaluator_gb300 as pe
    from helpers import assert_tree
    from oracle import instance as oinst
    from panoptic_evaluator_gb300 import synthetic, tuning
    images = synthetic.instance_batch(seed=21, images=6, side=(40, 90), preds=30)
    # Every other image padded to 16-byte rows (loaded by TMA), the rest staged.
    pad = lambda m, b: np.pad(m, ((0, 0), (0, 0), (0, (-m.shape[2]) % 16))) if b % 2 == 0 else m
    pm = [pad(i.pred_masks, b) for b, i in enumerate(images)]
    gm = [pad(i.gt_masks, b) for b, i in enumerate(images)]
    oracle = oinst.InstanceOracle(80)
    oracle.update(pm, [i.pred_classes for i in images], [i.scores for i in images], gm,
                  [i.gt_classes for i in images], [i.crowd for i in images])
    expected = oracle.compute()
    t = lambda x: torch.from_numpy(x).cuda()
    pred = pe.InstanceBatch([t(m) for m in pm], [t(i.pred_classes) for i in images], [t(i.scores) for i in images])
    target = pe.InstanceBatch([t(m) for m in gm], [t(i.gt_classes) for i in images],
                              crowd=[t(i.crowd) for i in images])
    ev = pe.InstanceEvaluator(80)
    result = tuning.tune_contract(ev, pred, target, repeats=2)
    key = result["tma_bucket"]
    try:
        assert 0 < key < 10 and len(result["candidates"]) == len(tuning.CONTRACT_TMA_COSTS)
        assert tuning.contract_cost(key) == result["tma_cost"]
        for cost in tuning.CONTRACT_TMA_COSTS:
            tuning.register_contract(key, cost)
            ev.reset()
            ev.update(pred, target)
            assert_tree(ev.compute(), expected)
    finally:
        tuning.forget_contract(key)
