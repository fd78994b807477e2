"""Replica merge of evaluator state (CPU): host merge rules and a gloo world of two ranks."""

import os
import socket

import numpy as np
import pytest
import torch
import torch.multiprocessing as mp

from oracle import instance as oinst
from oracle import panoptic as opan
from panoptic_evaluator_gb300 import distributed

C = 5
ISTHING = [True, True, True, False, False]


def panoptic_images():
    from panoptic_evaluator_gb300 import synthetic
    return synthetic.voronoi_batch(seed=21, B=6, H=40, W=48, sites=10, S=16, num_classes=C, things=3)


def instance_images():
    from panoptic_evaluator_gb300 import synthetic
    return synthetic.instance_batch(seed=22, images=6, side=(24, 40), num_classes=C, gt_range=(1, 6), preds=8)


def oracle_state(pan_idx, inst_idx):
    """State dict (GPU evaluator keys, CPU tensors) of the oracle over the given images."""
    p = panoptic_images()
    po = opan.PanopticOracle(C, ISTHING)
    if len(pan_idx):
        idx = list(pan_idx)
        po.update(p.pred[idx], p.pc[idx], p.gt[idx], p.gc[idx], p.crowd[idx])
    images = [instance_images()[i] for i in inst_idx]
    io = oinst.InstanceOracle(C)
    if images:
        io.update([i.pred_masks for i in images], [i.pred_classes for i in images], [i.scores for i in images],
                  [i.gt_masks for i in images], [i.gt_classes for i in images], [i.crowd for i in images])
    state = {f"panoptic/{k}": torch.from_numpy(np.asarray(getattr(po, k)).copy())
             for k in ("tp", "fp", "fn", "iou_sum", "confusion")}
    state["instance/counts"] = torch.from_numpy(io.counts.copy())
    recs = io.records
    cat = (lambda j, dt: np.concatenate([r[j] for r in recs]).astype(dt)) if recs else \
        (lambda j, dt: np.zeros(0, dt))
    state["instance/records.scores"] = torch.from_numpy(cat(0, np.float64))
    state["instance/records.classes"] = torch.from_numpy(cat(1, np.int32))
    state["instance/records.ranks"] = torch.from_numpy(cat(2, np.int32))
    flags = np.concatenate([r[3] for r in recs], axis=1).T.astype(np.int8) if recs else np.zeros((0, 40), np.int8)
    state["instance/records.flags"] = torch.from_numpy(np.ascontiguousarray(flags))
    return state, po, io


def instance_compute(state):
    flags = state["instance/records.flags"].numpy().T
    scores = state["instance/records.scores"].numpy()
    order = oinst.score_order(scores)
    precision, recall = oinst.accumulate(state["instance/records.classes"].numpy()[order],
                                         state["instance/records.ranks"].numpy()[order], flags[:, order],
                                         state["instance/counts"].numpy())
    return oinst.summarize(precision, recall)


def check_against_full(merged):
    full, po, io = oracle_state(range(6), range(6))
    for key, value in full.items():
        if key.endswith("iou_sum"):
            np.testing.assert_allclose(merged[key].numpy(), value.numpy(), rtol=1e-12, atol=1e-12)
        else:
            np.testing.assert_array_equal(merged[key].numpy(), value.numpy(), err_msg=key)
    got, want = instance_compute(merged), io.compute()
    for key in want:
        np.testing.assert_allclose(np.asarray(got[key]), np.asarray(want[key]), rtol=1e-12, atol=1e-12,
                                   err_msg=key)


def test_merge_rules():
    f64 = dict(dtype=torch.float64)
    a = {"tp": torch.tensor([1, 2]), "iou_sum": torch.tensor([0.1, 0.2], **f64),
         "records.scores": torch.tensor([0.5], **f64), "records.flags": torch.zeros((1, 40), dtype=torch.int8)}
    b = {"tp": torch.tensor([3, 4]), "iou_sum": torch.tensor([0.3, 0.4], **f64),
         "records.scores": torch.tensor([0.7, 0.9], **f64), "records.flags": torch.ones((2, 40), dtype=torch.int8)}
    m = distributed.merge_states([a, b])
    assert m["tp"].tolist() == [4, 6]
    assert m["iou_sum"].tolist() == [0.1 + 0.3, 0.2 + 0.4]
    assert m["records.scores"].tolist() == [0.5, 0.7, 0.9]
    assert m["records.flags"].shape == (3, 40) and m["records.flags"][1:].all()
    assert a["tp"].tolist() == [1, 2]  # inputs untouched
    with pytest.raises(ValueError):
        distributed.merge_states([a, {"tp": a["tp"]}])


def test_host_merge_of_oracle_halves_equals_full():
    first, _, _ = oracle_state(range(3), range(3))
    second, _, _ = oracle_state(range(3, 6), range(3, 6))
    check_against_full(distributed.merge_states([first, second]))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    torch.distributed.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                                         world_size=world)
    try:
        share = [list(range(r * 6 // world, (r + 1) * 6 // world)) for r in range(world)][rank]
        state, _, _ = oracle_state(share, share)
        merged = distributed.all_reduce_states(state)
        torch.save(merged, os.path.join(out, f"rank{rank}.pt"))
    finally:
        torch.distributed.destroy_process_group()


@pytest.mark.parametrize("world", [2])
def test_gloo_ranks_merge_to_the_full_state(tmp_path, world):
    mp.spawn(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    states = [torch.load(tmp_path / f"rank{r}.pt") for r in range(world)]
    for state in states[1:]:  # every rank holds the same merged state, bit for bit
        for key in states[0]:
            assert torch.equal(state[key], states[0][key]), key
    check_against_full(states[0])
