"""Parity with the oracle at the benchmark configurations' own sizes.

Each test evaluates a seeded synthetic workload of one configuration's shapes
and value distributions on the GPU and compares the whole result with the
oracle: integer counts, confusion, flags and ranks exactly, FP64 metrics
within 1e-12 (``helpers.RTOL`` / ``ATOL``).

* PanopticEvaluator / panoptic_quality on COCO-shape batches: B = 16 images of
  480-640 per side on a 640 x 640 canvas, up to 101 / 121 slots, 133 classes
  (``evaluator.py:291-544``);
* InstanceEvaluator on 16 images of 480-640 per side, 1-50 targets and 100
  predictions each, 80 classes (``instance.py:172-227``);
* SegmentationEvaluator on 48 uneven images with sides 320-1024, 10-150 slots
  and 5-100 detections (``combined.py:63-167``), batched and per call;
* segmentation_prefixes on 8 images of 256-1024 per side with 64 masks,
  checkpoints 8..64 (``prefix.py:11-122``);
* the reward server on a mix of those panoptic_quality and prefix requests.
"""

import multiprocessing as mp
from functools import partial

import numpy as np
import pytest
import torch

from helpers import assert_tree, cuda
from oracle import combined as ocomb
from oracle import instance as oinst
from oracle import panoptic as opan
from oracle import prefix as opre

pytestmark = pytest.mark.gpu

C, THINGS = 133, 80
ISTHING = [c < THINGS for c in range(C)]
POINTS = list(range(8, 65, 8))


@pytest.fixture(scope="module")
def pe():
    import panoptic_evaluator_gb300 as pe
    return pe


@pytest.fixture(scope="module")
def pool():
    # Spawned workers generate the inputs; no CUDA state is forked.
    with mp.get_context("spawn").Pool(8) as workers:
        yield workers


def test_coco_panoptic_batch_of_16(pe):
    from panoptic_evaluator_gb300 import synthetic
    a = synthetic.coco_panoptic_batch(seed=21)
    assert a.gt.shape == (16, 640, 640)
    oracle = opan.PanopticOracle(C, a.isthing)
    oracle.update(a.pred, a.pc, a.gt, a.gc, a.crowd)
    pred, target = pe.PanopticBatch(cuda(a.pred), cuda(a.pc)), pe.PanopticBatch(cuda(a.gt), cuda(a.gc), cuda(a.crowd))
    for validate in (True, False):
        ev = pe.PanopticEvaluator(C, isthing=ISTHING, validate=validate)
        ev.update(pred, target)
        assert_tree(ev.compute(), oracle.compute())
    stats = pe.panoptic_quality(pred, target, C, return_stats=True)
    assert_tree(stats, opan.panoptic_quality(a.pred, a.pc, a.gt, a.gc, a.crowd, C, return_stats=True))
    assert_tree(pe.panoptic_quality(pred, target, C), opan.panoptic_quality(a.pred, a.pc, a.gt, a.gc, a.crowd, C))


def test_coco_instance_batch_of_16(pe, pool):
    from panoptic_evaluator_gb300 import synthetic
    images = pool.map(partial(synthetic.instance_one, 22), range(16), chunksize=1)
    assert all(len(i.pred_masks) == 100 and 480 <= i.pred_masks.shape[1] <= 640 for i in images)
    oracle = oinst.InstanceOracle(THINGS)
    oracle.update([i.pred_masks for i in images], [i.pred_classes for i in images], [i.scores for i in images],
                  [i.gt_masks for i in images], [i.gt_classes for i in images], [i.crowd for i in images])
    expected = oracle.compute()
    pred = pe.InstanceBatch([cuda(i.pred_masks) for i in images], [cuda(i.pred_classes) for i in images],
                            [cuda(i.scores) for i in images])
    target = pe.InstanceBatch([cuda(i.gt_masks) for i in images], [cuda(i.gt_classes) for i in images],
                              crowd=[cuda(i.crowd) for i in images])
    for validate in (True, False):
        ev = pe.InstanceEvaluator(THINGS, validate=validate)
        ev.update(pred, target)
        assert_tree(ev.compute(), expected)


def test_uneven_combined_batch_of_48(pe, pool):
    from panoptic_evaluator_gb300 import synthetic
    from panoptic_evaluator_gb300.ragged import SegmentationImages
    images = synthetic.segmentation_batch(seed=23, images=48, pool=pool)
    sides = np.array([i.target.shape for i in images])
    assert sides.min() >= 320 and sides.max() <= 1024
    parts = pool.map(ocomb.image_update, [(i.pred, i.pred_classes, i.det_masks, i.det_classes, i.scores, i.target,
                                           i.target_classes, i.crowd, C, ISTHING) for i in images])
    expected = ocomb.merge(parts, C, ISTHING).compute()
    arena = SegmentationImages([i.target for i in images], [i.target_classes for i in images],
                               [i.crowd for i in images], [i.pred for i in images], [i.pred_classes for i in images],
                               [i.det_masks for i in images], [i.det_classes for i in images],
                               [i.scores for i in images])
    for validate in (True, False):
        batched = pe.SegmentationEvaluator(C, isthing=ISTHING, validate=validate)
        batched.update_images(arena)
        assert_tree(batched.compute(), expected)
    per_call = pe.SegmentationEvaluator(C, isthing=ISTHING)
    for i in images:
        per_call.update(pe.PanopticBatch(cuda(i.pred[None]), cuda(i.pred_classes[None])),
                        pe.InstanceBatch([cuda(i.det_masks)], [cuda(i.det_classes)], [cuda(i.scores)]),
                        pe.PanopticBatch(cuda(i.target[None]), cuda(i.target_classes[None]), cuda(i.crowd[None])))
    assert_tree(per_call.compute(), expected)


def _prefix_expected(image):
    return opre.image_prefixes(image.target, image.target_classes, image.crowd, image.masks, image.classes,
                               np.array(ISTHING), C, np.array([0.5, 0.75]), set(POINTS))


def test_generation_prefixes_of_8_images(pe, pool):
    from panoptic_evaluator_gb300 import synthetic
    images = synthetic.prefix_batch(seed=24, images=8, masks=64, pool=pool)
    expected = pool.map(_prefix_expected, images)
    target = pe.PanopticBatch(cuda(np.stack([i.target for i in images])),
                              cuda(np.stack([i.target_classes for i in images])),
                              cuda(np.stack([i.crowd for i in images])))
    pred = pe.InstanceBatch([cuda(i.masks) for i in images], [cuda(i.classes) for i in images])
    for validate in (True, False):
        result = pe.segmentation_prefixes(pred, target, C, isthing=ISTHING, checkpoints=POINTS, validate=validate)
        assert_tree(result, expected)


def _pq_expected(image):
    return opan.panoptic_quality(image.pred[None], image.pred_classes[None], image.target[None],
                                 image.target_classes[None], image.crowd[None], C)[0]


def test_reward_server_mix_at_full_size(pe, pool):
    """PQ requests (sides 256-1024) and 64-mask prefix requests, served together, each equal to the oracle."""
    from panoptic_evaluator_gb300 import synthetic
    from panoptic_evaluator_gb300.serving import PanopticRequest, PrefixRequest, RewardServer, serve
    panoptic = pool.map(partial(synthetic.segmentation_one, 25, side=(256, 1024), slots=(10, 100), dets=(0, 0)),
                        range(24))
    prefixes = pool.map(partial(synthetic.prefix_one, 26, side=(256, 1024), masks=64, slots=101), range(8))
    pq_expected = pool.map(_pq_expected, panoptic)
    prefix_expected = pool.map(_prefix_expected, prefixes)
    requests = [PanopticRequest(i.pred, i.pred_classes, i.target, i.target_classes, i.crowd) for i in panoptic]
    requests += [PrefixRequest(i.masks, i.classes, i.target, i.target_classes, i.crowd, checkpoints=POINTS)
                 for i in prefixes]
    order = np.random.default_rng(27).permutation(len(requests))
    arrivals = np.cumsum(np.random.default_rng(28).exponential(1 / 2000.0, len(requests)))
    with RewardServer(C, isthing=ISTHING, memory_budget=4 << 30, max_batch=16) as server:
        responses, _ = serve(server, [requests[i] for i in order], arrivals)
    for response, index in zip(responses, order):
        if index < len(panoptic):
            np.testing.assert_allclose(response.values["pq"], pq_expected[index], rtol=1e-12, atol=1e-12)
        else:
            expected = prefix_expected[index - len(panoptic)]
            assert_tree(response.values["snapshots"],
                        [{k: s[k] for k in ("All", "Things", "Stuff", "prefix", "miou", "instance")}
                         for s in expected])
    torch.cuda.synchronize()
