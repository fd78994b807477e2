"""Replicas on one GPU: merged state of evaluators over disjoint image shares equals one evaluator over all."""

import pytest
import torch

from helpers import assert_tree

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pe():
    import panoptic_evaluator_gb300 as pe
    return pe


def segmentation(pe, images, evaluator):
    from panoptic_evaluator_gb300.ragged import SegmentationImages
    arena = SegmentationImages([i.target for i in images], [i.target_classes for i in images],
                               [i.crowd for i in images], [i.pred for i in images], [i.pred_classes for i in images],
                               [i.det_masks for i in images], [i.det_classes for i in images],
                               [i.scores for i in images])
    evaluator.update_images(arena)
    return evaluator


def test_segmentation_replicas_merge_to_single_evaluator(pe):
    from panoptic_evaluator_gb300 import distributed, synthetic
    images = synthetic.segmentation_batch(seed=31, images=9, side=(40, 120), slots=(10, 40), dets=(0, 12))
    isthing = [c < 80 for c in range(133)]
    single = segmentation(pe, images, pe.SegmentationEvaluator(133, isthing=isthing))
    shares = [images[:3], images[3:7], images[7:]]  # contiguous split, one replica per share
    states = [segmentation(pe, share, pe.SegmentationEvaluator(133, isthing=isthing)).state_dict()
              for share in shares]
    merged = pe.SegmentationEvaluator(133, isthing=isthing).load_state_dict(distributed.merge_states(states))
    assert_tree(merged.compute(), single.compute())
    for key, value in single.state_dict().items():
        if value.is_floating_point() and "iou_sum" in key:
            torch.testing.assert_close(merged.state_dict()[key], value, rtol=1e-12, atol=1e-12)
        else:
            assert torch.equal(merged.state_dict()[key], value), key


def test_instance_state_round_trip(pe):
    from panoptic_evaluator_gb300 import synthetic
    images = synthetic.instance_batch(seed=32, images=3, side=(30, 50), gt_range=(1, 8), preds=12)
    pred = pe.InstanceBatch([torch.from_numpy(i.pred_masks).cuda() for i in images],
                            [torch.from_numpy(i.pred_classes).cuda() for i in images],
                            [torch.from_numpy(i.scores).cuda() for i in images])
    target = pe.InstanceBatch([torch.from_numpy(i.gt_masks).cuda() for i in images],
                              [torch.from_numpy(i.gt_classes).cuda() for i in images],
                              crowd=[torch.from_numpy(i.crowd).cuda() for i in images])
    ev = pe.InstanceEvaluator(80).update(pred, target)
    copy = pe.InstanceEvaluator(80).load_state_dict({k: v.cpu() for k, v in ev.state_dict().items()})
    assert_tree(copy.compute(), ev.compute(), exact_float=True)
    with pytest.raises(ValueError):
        copy.load_state_dict({**ev.state_dict(), "counts": torch.zeros((3, 4), dtype=torch.int64)})
