"""COCO panoptic PNG pixels on the GPU: RGB -> IDs -> slots against the oracle and the integer-ID path."""

import numpy as np
import pytest
import torch

from helpers import assert_tree
from oracle import panoptic as opan

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pe():
    import panoptic_evaluator_gb300 as pe
    return pe


def coco_like(rng, B, H, W, segments, void=0.1):
    """ID maps with `segments` random IDs below 2^24 per image, plus segments_info."""
    maps = np.zeros((B, H, W), np.int64)
    infos = []
    for b in range(B):
        ids = rng.choice(np.arange(1, 2**24), segments, replace=False)
        maps[b] = rng.choice(ids, (H, W))
        maps[b][rng.random((H, W)) < void] = 0
        infos.append([dict(id=int(i), category_id=int(rng.integers(1, 4)), iscrowd=int(rng.random() < 0.1))
                      for i in rng.permutation(ids)])
    return maps, infos


@pytest.mark.parametrize("B,H,W,S", [(2, 7, 9, 3), (3, 64, 64, 20), (1, 481, 483, 300), (2, 1024, 1024, 60)])
def test_rgb_from_coco_matches_integer_ids_and_oracle(pe, B, H, W, S):
    rng = np.random.default_rng(H * W + S)
    maps, infos = coco_like(rng, B, H, W, S)
    rgb = torch.from_numpy(opan.encode_rgb(maps)).cuda()
    ids = torch.from_numpy(maps).cuda()
    np.testing.assert_array_equal(pe.evaluator.decode_rgb(rgb).cpu().numpy(), maps)
    from_rgb = pe.PanopticBatch.from_coco(rgb, infos, [1, 2, 3])
    from_ids = pe.PanopticBatch.from_coco(ids, infos, [1, 2, 3])
    assert torch.equal(from_rgb.segment_map, from_ids.segment_map)
    t_ids, t_slots, _, _ = opan.from_coco(maps, infos, [1, 2, 3])
    np.testing.assert_array_equal(from_rgb.segment_map.cpu().numpy(), opan.pack(maps, t_ids, t_slots))
    lazy = pe.PanopticBatch.from_coco(rgb, infos, [1, 2, 3], compact=False)
    assert lazy.segment_map.dtype == torch.int32 and torch.equal(lazy.segment_map.long(), ids)
    assert torch.equal(lazy.compact().segment_map, from_ids.segment_map)


def test_rgb_batches_evaluate_like_integer_batches(pe):
    rng = np.random.default_rng(7)
    maps, infos = coco_like(rng, 2, 40, 50, 12)
    pred = maps.copy()
    pred[:, :5] = 0
    rgb_gt, rgb_pred = (torch.from_numpy(opan.encode_rgb(m)).cuda() for m in (maps, pred))
    pred_infos = [[{**e, "iscrowd": 0} for e in info] for info in infos]
    results = []
    for gt_maps, pred_maps in ((rgb_gt, rgb_pred), (torch.from_numpy(maps).cuda(), torch.from_numpy(pred).cuda())):
        ev = pe.PanopticEvaluator(3)
        ev.update(pe.PanopticBatch.from_coco(pred_maps, pred_infos, [1, 2, 3]),
                  pe.PanopticBatch.from_coco(gt_maps, infos, [1, 2, 3]))
        results.append(ev.compute())
    assert_tree(results[0], results[1], exact_float=True)


def test_rgb_absent_ids_and_with_maps(pe):
    rng = np.random.default_rng(8)
    maps, infos = coco_like(rng, 1, 16, 16, 5)
    rgb = torch.from_numpy(opan.encode_rgb(maps)).cuda()
    batch = pe.PanopticBatch.from_coco(rgb, infos, [1, 2, 3], compact=False)
    other = maps.copy()
    other[0, 0, 0] = int(infos[0][0]["id"])
    again = batch.with_maps(torch.from_numpy(opan.encode_rgb(other)).cuda())
    assert again.segment_map[0, 0, 0].item() == infos[0][0]["id"]
    broken = maps.copy()
    broken[0, 3, 3] = 2**24 - 1 if 2**24 - 1 not in [e["id"] for e in infos[0]] else 2**24 - 2
    with pytest.raises(ValueError):
        pe.PanopticBatch.from_coco(torch.from_numpy(opan.encode_rgb(broken)).cuda(), infos, [1, 2, 3])
    with pytest.raises(ValueError):
        pe.PanopticBatch(torch.zeros((1, 4, 4), dtype=torch.int32, device="cuda"),
                         torch.full((1, 2), -1, dtype=torch.int32, device="cuda")).with_maps(rgb)
