"""Tensor-core mask contraction (pe_inst_contract): exact pixel counts for every detection x target pair."""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def inst():
    from panoptic_evaluator_gb300 import instance
    return instance


def reference(pm, gm):
    a = pm.reshape(pm.shape[0], pm.shape[1] * pm.shape[2]).astype(np.float64)
    b = gm.reshape(gm.shape[0], gm.shape[1] * gm.shape[2]).astype(np.float64)
    return (a @ b.T).astype(np.int64), a.sum(1).astype(np.int64), b.sum(1).astype(np.int64)


def check(inst, images):
    pred = [torch.from_numpy(p).cuda() for p, _ in images]
    gt = [torch.from_numpy(g).cuda() for _, g in images]
    got = inst.pairwise_intersections(pred, gt)
    for (p, g), (inter, pa, ga) in zip(images, got):
        e_inter, e_pa, e_ga = reference(p, g)
        np.testing.assert_array_equal(inter.cpu().numpy(), e_inter)
        np.testing.assert_array_equal(pa.cpu().numpy(), e_pa)
        np.testing.assert_array_equal(ga.cpu().numpy(), e_ga)


def random_masks(rng, n, h, w, density):
    return rng.random((n, h, w)) < density


@pytest.mark.parametrize("d,g,h,w", [(5, 3, 7, 9), (1, 1, 1, 1), (100, 50, 97, 83), (127, 63, 64, 64),
                                     (128, 64, 17, 19), (130, 70, 33, 65), (300, 10, 20, 21), (7, 200, 41, 43),
                                     (0, 5, 40, 40), (5, 0, 40, 40), (12, 9, 211, 307)])
def test_random_masks_all_shapes(inst, d, g, h, w):
    rng = np.random.default_rng(d * 1000 + g + h)
    images = [(random_masks(rng, d, h, w, 0.3), random_masks(rng, g, h, w, 0.5)),
              (random_masks(rng, d, h, w, 0.02), random_masks(rng, g, h, w, 0.9))]
    check(inst, images)


def test_full_masks_reach_large_counts(inst):
    """All-ones 640 x 640 masks: every count is 409,600 (409,600 x 2^-18 in one fp32 accumulator)."""
    ones = np.ones((9, 640, 640), bool)
    check(inst, [(ones, ones[:4])])


def test_unaligned_row_starts_and_uneven_batch(inst):
    rng = np.random.default_rng(3)
    base = rng.random((41, 29, 31)) < 0.4  # 899-byte rows: every row starts at a different offset mod 16
    gt = torch.from_numpy(rng.random((6, 29, 31)) < 0.6).cuda()
    dev = torch.from_numpy(base).cuda()
    views = [dev[1:], dev[3:17], dev[5:6]]  # contiguous views starting mid-allocation
    got = inst.pairwise_intersections(views, [gt, gt[2:], gt[:1]])
    for view, target, (inter, pa, ga) in zip(views, [gt, gt[2:], gt[:1]], got):
        e_inter, e_pa, e_ga = reference(view.cpu().numpy(), target.cpu().numpy())
        np.testing.assert_array_equal(inter.cpu().numpy(), e_inter)
        np.testing.assert_array_equal(pa.cpu().numpy(), e_pa)
        np.testing.assert_array_equal(ga.cpu().numpy(), e_ga)


def test_coco_shaped_instance_masks(inst):
    from panoptic_evaluator_gb300 import synthetic
    images = synthetic.instance_batch(seed=8, images=3)
    check(inst, [(im.pred_masks, im.gt_masks) for im in images])


def test_instance_evaluator_same_with_both_contractions(inst):
    import panoptic_evaluator_gb300 as pe
    from panoptic_evaluator_gb300 import synthetic
    images = synthetic.instance_batch(seed=9, images=4)
    pred = pe.InstanceBatch([torch.from_numpy(i.pred_masks).cuda() for i in images],
                            [torch.from_numpy(i.pred_classes).cuda() for i in images],
                            [torch.from_numpy(i.scores).cuda() for i in images])
    target = pe.InstanceBatch([torch.from_numpy(i.gt_masks).cuda() for i in images],
                              [torch.from_numpy(i.gt_classes).cuda() for i in images],
                              crowd=[torch.from_numpy(i.crowd).cuda() for i in images])
    results = {}
    saved = inst.CONTRACTION
    try:
        for method in ("tensor", "popcount"):
            inst.CONTRACTION = method
            ev = pe.InstanceEvaluator(80)
            ev.update(pred, target)
            results[method] = ev.compute()
    finally:
        inst.CONTRACTION = saved
    for key, value in results["tensor"].items():
        torch.testing.assert_close(value, results["popcount"][key], rtol=0, atol=0, equal_nan=True)


@pytest.mark.parametrize("h,w,density", [(1024, 1024, 0.5), (1024, 1024, 0.97), (2048, 2048, 0.5),
                                         (2048, 2048, 0.97), (2047, 2049, 0.9), (2304, 2304, 0.75)])
def test_large_random_counts_are_exact(inst, h, w, density):
    """Counts from 2^17 up to the 2^22-pixel read-back bound (and past it: 2304^2 spans two segments).

    Random masks make every 32-byte K step add an arbitrary number of 2^-18
    products, odd or even, to accumulators that already hold up to 2^22 of
    them: a tensor core that dropped low accumulator bits would miscount here.
    2047 x 2049 puts every mask row at a different byte offset.
    """
    rng = np.random.default_rng(h * 7 + w + int(density * 100))
    pred = random_masks(rng, 8, h, w, density)
    gt = np.concatenate([random_masks(rng, 3, h, w, density), np.ones((1, h, w), bool)])
    check(inst, [(pred, gt)])


def test_odd_increment_every_k_step(inst):
    """Each prediction row sets 31 of every 32 bytes (one K step of the MMA): every step adds an odd count.

    Against an all-ones target the count climbs to 31/32 of 2^22 in odd steps of
    31 x 2^-18 within one accumulator, so any truncated low bit shows.
    """
    h = w = 2048
    pixels = np.arange(h * w)
    pred = np.stack([(pixels + shift) % 32 != 0 for shift in (0, 5, 17, 31)]).reshape(4, h, w)
    gt = np.stack([np.ones(h * w, bool), (pixels % 3) != 0]).reshape(2, h, w)
    check(inst, [(pred, gt)])


@pytest.mark.parametrize("direct", [False, True])
def test_direct_and_staged_rows_in_one_batch(inst, direct):
    """Images with rows on 16-byte boundaries (copied straight into the operand tiles) between images
    whose rows start at other offsets (staged and re-aligned), so CTAs cross between both kinds of block.

    Sizes: 64 x 64, 48 x 100 (4800 pixels: a 704-pixel tail chunk ending mid-stage) and 12 x 12 on
    16-byte boundaries; 20 x 21 (420-byte rows) and 29 x 31 (899) off them; views starting one row
    into an allocation (256 bytes: still aligned; 420 bytes: not).
    """
    rng = np.random.default_rng(11 if direct else 12)
    shapes = [(64, 64), (20, 21), (29, 31), (48, 100), (20, 21), (64, 64), (29, 31), (12, 12)]
    images = []
    for i, (h, w) in enumerate(shapes):
        d, g = (130, 70) if i % 3 == 0 else (40 + i, 9 + 2 * i)
        images.append((random_masks(rng, d, h, w, 0.3 + 0.05 * i), random_masks(rng, g, h, w, 0.6)))
    pred = [torch.from_numpy(p).cuda() for p, _ in images]
    gt = [torch.from_numpy(g).cuda() for _, g in images]
    for h, w in ((16, 16), (20, 21)):
        base = torch.from_numpy(random_masks(rng, 33, h, w, 0.5)).cuda()
        pred.append(base[1:])
        gt.append(base[3:9].clone())
    got = inst.pairwise_intersections(pred, gt, direct=direct)
    for p, g, (inter, pa, ga) in zip(pred, gt, got):
        e_inter, e_pa, e_ga = reference(p.cpu().numpy(), g.cpu().numpy())
        np.testing.assert_array_equal(inter.cpu().numpy(), e_inter)
        np.testing.assert_array_equal(pa.cpu().numpy(), e_pa)
        np.testing.assert_array_equal(ga.cpu().numpy(), e_ga)
