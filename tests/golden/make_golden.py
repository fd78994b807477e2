"""Generate golden vectors by running the reference's own CPU implementation.

Run where a reference checkout is available, naming its path:

    python tests/golden/make_golden.py --reference <path to the reference checkout>

It imports ``panoptic_evaluator`` from that checkout (CPU tensors only; the
reference's CUDA extension is not needed), evaluates seeded inputs and writes
``tests/golden/*.npz``. Each file holds ``in/...`` input arrays and
``out/...`` reference outputs. ``tests/test_oracle.py`` replays the inputs
through ``oracle/`` and requires the same outputs, which pins the oracle to
the reference. The fixtures are committed; the reference is not needed to run
the tests.
"""

from __future__ import annotations

import argparse
import sys
from pathlib import Path

import numpy as np
import torch

HERE = Path(__file__).resolve().parent


def flatten(prefix, value, out):
    if isinstance(value, dict):
        for key, item in value.items():
            flatten(f"{prefix}/{key}", item, out)
    elif isinstance(value, (list, tuple)):
        out[f"{prefix}/__len__"] = np.array(len(value))
        for index, item in enumerate(value):
            flatten(f"{prefix}/{index}", item, out)
    elif isinstance(value, torch.Tensor):
        out[prefix] = value.detach().cpu().numpy()
    elif value is None:
        out[f"{prefix}/__none__"] = np.array(0)
    else:
        out[prefix] = np.asarray(value)


def save(name, inputs, outputs):
    arrays = {}
    flatten("in", inputs, arrays)
    flatten("out", outputs, arrays)
    np.savez_compressed(HERE / f"{name}.npz", **arrays)


def panoptic_cases(pe):
    """PanopticEvaluator.update/compute on CPU (evaluator.py:246-468)."""
    cases = []
    g = torch.Generator().manual_seed(857)
    # Known-answer shapes from the reference tests, as compact slots.
    kat = [
        ([[[0, 1, 1, 2]]], [[-1, 0, 1]], None, [[[0, 1, 1, 2]]], [[-1, 0, 1]]),
        ([[[1, 1, 1, 1]]], [[-1, 0]], None, [[[1, 1, 0, 0]]], [[-1, 0]]),
        ([[[1, 1, 1]]], [[-1, 0]], None, [[[1, 1, 0]]], [[-1, 0]]),
        ([[[1, 0, 0, 0]]], [[-1, 0]], None, [[[1, 1, 1, 1]]], [[-1, 0]]),
        ([[[1, 1, 0]]], [[-1, 0]], [[False, True]], [[[1, 1, 1]]], [[-1, 0]]),
        ([[[1, 1, 1, 1]]], [[-1, 0]], [[False, True]], [[[1, 1, 1, 1]]], [[-1, 1]]),
        ([[[0, 0, 1, 1]]], [[-1, 1]], None, [[[1, 1, 1, 1]]], [[-1, 0]]),
        ([[[1, 1, 2, 2]]], [[-1, 0, 1]], None, [[[1, 0, 1, 2]]], [[-1, 0, 1]]),
    ]
    for gt, gc, crowd, pred, pc in kat:
        cases.append(dict(gt=torch.tensor(gt, dtype=torch.int32), gc=torch.tensor(gc, dtype=torch.int32),
                          crowd=None if crowd is None else torch.tensor(crowd),
                          pred=torch.tensor(pred, dtype=torch.int32), pc=torch.tensor(pc, dtype=torch.int32),
                          C=3, isthing=[True, False, True], validate=True))
    # Varied capacities with random metadata (validation off), crowd and void.
    for G, P in ((1, 1), (2, 3), (65, 97), (257, 513), (97, 65)):
        gt = torch.randint(G, (3, 31, 47), generator=g, dtype=torch.int32)
        pred = torch.randint(P, gt.shape, generator=g, dtype=torch.int32)
        gc = torch.randint(5, (3, G), generator=g, dtype=torch.int32)
        pc = torch.randint(5, (3, P), generator=g, dtype=torch.int32)
        gc[:, 0] = pc[:, 0] = -1
        crowd = torch.rand((3, G), generator=g) < .25
        crowd[:, 0] = False
        if G == 65:
            pred = gt.clone()
            pc[:, :G] = gc
            pc[:, G:] = -1
            pred[:, ::5, :] = 0
        cases.append(dict(gt=gt, gc=gc, crowd=crowd, pred=pred, pc=pc, C=5,
                          isthing=[True, True, False, True, False], validate=False))
    # Coherent blocks with valid metadata (validation on), as a perturbed copy.
    for B, H, W, S, C in ((2, 24, 40, 9, 4), (4, 33, 17, 21, 7)):
        gt = (torch.arange(H)[:, None] // 6 * 7 + torch.arange(W)[None] // 5) % (S - 1) + 1
        gt = gt[None].repeat(B, 1, 1).int()
        gt[:, ::7] = 0
        pred = gt.clone()
        noise = torch.rand(gt.shape, generator=g) < .2
        pred[noise] = torch.randint(S, (int(noise.sum()),), generator=g, dtype=torch.int32)
        gc = torch.randint(C, (B, S), generator=g, dtype=torch.int32)
        pc = gc.clone()
        flip = torch.rand((B, S), generator=g) < .2
        pc[flip] = torch.randint(C, (int(flip.sum()),), generator=g, dtype=torch.int32)
        gc[:, 0] = pc[:, 0] = -1
        for maps, classes in ((gt, gc), (pred, pc)):
            present = torch.stack([torch.bincount(m.flatten().long(), minlength=S) > 0 for m in maps])
            classes[~present] = -1
            classes[:, 0] = -1
        crowd = (torch.rand((B, S), generator=g) < .15) & (gc >= 0)
        cases.append(dict(gt=gt, gc=gc, crowd=crowd, pred=pred, pc=pc, C=C,
                          isthing=[i % 2 == 0 for i in range(C)], validate=True))
    outputs = []
    for case in cases:
        ev = pe.PanopticEvaluator(case["C"], isthing=case["isthing"], device="cpu", validate=case["validate"])
        ev.update(pe.PanopticBatch(case["pred"], case["pc"]),
                  pe.PanopticBatch(case["gt"], case["gc"], case["crowd"]))
        outputs.append(ev.compute())
    save("panoptic", cases, outputs)


def original_id_cases(pe):
    """from_coco + compact on original IDs (evaluator.py:33-158)."""
    large = 2**40 + 17
    gt = torch.tensor([[[0, large, large, 1234], [7, 7, large, 1234]],
                       [[99, 99, 0, 0], [0, 0, 0, 0]]], dtype=torch.int64)
    pred = torch.tensor([[[123, 123, 123, 123], [900, 900, 123, 123]],
                         [[321, 321, 0, 0], [0, 0, 0, 0]]], dtype=torch.int64)
    gi = [[{"id": 1234, "category_id": 7, "iscrowd": 1},
           {"id": large, "category_id": 7, "iscrowd": 1},
           {"id": 7, "category_id": 42}], [{"id": 99, "category_id": 91}]]
    pi = [[{"id": 900, "category_id": 42}, {"id": 123, "category_id": 7}],
          [{"id": 321, "category_id": 91}]]
    cats = (7, 42, 91)
    target = pe.PanopticBatch.from_coco(gt, gi, cats, compact=False)
    prediction = pe.PanopticBatch.from_coco(pred, pi, cats, compact=False)
    ev = pe.PanopticEvaluator(3, device="cpu")
    ev.update(prediction.compact(), target.compact())
    tables = {name: getattr(target, name) for name in ("classes", "crowd", "lookup_ids", "lookup_slots")}
    ptables = {name: getattr(prediction, name) for name in ("classes", "crowd", "lookup_ids", "lookup_slots")}
    save("original_ids",
         dict(gt=gt, pred=pred, target=tables, prediction=ptables,
              gt_compact=target.compact().segment_map, pred_compact=prediction.compact().segment_map),
         ev.compute())


def reward_cases(pe):
    """panoptic_quality on CPU (evaluator.py:471-544)."""
    gt = torch.tensor([[[1, 1, 1, 1]], [[1, 1, 1, 0]], [[1, 0, 0, 0]], [[2, 2, 0, 0]],
                       [[0, 0, 0, 0]], [[1, 1, 1, 1]], [[1, 1, 1, 1]], [[1, 1, 2, 2]]], dtype=torch.int32)
    pred = torch.tensor([[[1, 1, 0, 0]], [[1, 1, 0, 0]], [[1, 1, 1, 1]], [[2, 2, 2, 2]],
                         [[0, 0, 0, 0]], [[0, 0, 0, 0]], [[1, 1, 1, 1]], [[1, 1, 2, 2]]], dtype=torch.int32)
    gc = torch.tensor([[-1, 0, -1], [-1, 0, -1], [-1, 0, -1], [-1, -1, 1], [-1, -1, -1], [-1, 0, -1],
                       [-1, 0, -1], [-1, 0, 2]], dtype=torch.int32)
    pc = torch.tensor([[-1, 0, 2]] * 8, dtype=torch.int32)
    pc[3, 2] = 1
    crowd = torch.zeros_like(gc, dtype=torch.bool)
    crowd[3, 2] = True
    cases = [dict(gt=gt, pred=pred, gc=gc, pc=pc, crowd=crowd, C=4)]
    g = torch.Generator().manual_seed(19)
    for _ in range(6):
        gt = torch.randint(0, 7, (5, 9, 13), generator=g).int()
        pred = gt.clone()
        pred[:, ::3] = torch.randint(0, 9, (5, 3, 13), generator=g).int()
        gc = torch.randint(0, 4, (5, 7), generator=g).int()
        pc = torch.cat((gc.clone(), torch.zeros((5, 2), dtype=torch.int32)), 1)
        gc[:, 0] = pc[:, 0] = -1
        crowd = torch.rand((5, 7), generator=g) < .25
        crowd[:, 0] = False
        cases.append(dict(gt=gt, pred=pred, gc=gc, pc=pc, crowd=crowd, C=5))
    outputs = []
    for case in cases:
        t = pe.PanopticBatch(case["gt"], case["gc"], case["crowd"])
        p = pe.PanopticBatch(case["pred"], case["pc"])
        outputs.append(dict(pq=pe.panoptic_quality(p, t, case["C"], validate=False),
                            stats=pe.panoptic_quality(p, t, case["C"], validate=False, return_stats=True)))
    save("reward", cases, outputs)


def matcher_cases():
    """Adversarial COCO matcher inputs (instance.py:267-297), as in the reference tests."""
    from panoptic_evaluator.instance import _match_ious_cpu
    g = torch.Generator().manual_seed(802)
    cases, outputs = [], []
    for D, G, C in ((0, 65, 3), (105, 0, 3), (113, 97, 3), (131, 137, 1), (17, 99, 1), (40, 40, 4)):
        pc = torch.randint(C, (D,), generator=g, dtype=torch.int32)
        gc = torch.randint(C, (G,), generator=g, dtype=torch.int32)
        crowd = torch.rand(G, generator=g) < 0.2
        choices = torch.tensor([0.0, 1.0, 1024.0, 1025.0, 9216.0, 9217.0, 1e10, 1e10 + 1], dtype=torch.float64)
        ga = choices[torch.randint(len(choices), (G,), generator=g)]
        pairs = torch.ones((D, G), dtype=torch.int64)
        pixel_ga = torch.full((G,), 2.0, dtype=torch.float64)
        pixel_pa = torch.ones(D, dtype=torch.float64)
        if D in (17, 40):
            pairs = torch.randint(0, 11, (D, G), generator=g)
            pixel_ga.fill_(10.0)
            pixel_pa = choices[torch.randint(len(choices), (D,), generator=g)].clamp_min(10.0) if D == 40 \
                else pixel_pa.fill_(10.0)
        union = torch.where(crowd[None], pixel_pa[:, None], pixel_pa[:, None] + pixel_ga[None] - pairs)
        ious = pairs.double() / union.clamp_min(1)
        status, ranks, counts = _match_ious_cpu(ious, pc, gc, pixel_pa, crowd, ga, C)
        cases.append(dict(pairs=pairs, pc=pc, gc=gc, pa=pixel_pa, ga=pixel_ga, crowd=crowd, areas=ga, C=C))
        outputs.append(dict(status=status, ranks=ranks, counts=counts))
    save("matcher", cases, outputs)


def instance_cases(pe):
    """InstanceEvaluator update/compute on CPU (instance.py:46-331)."""
    g = torch.Generator().manual_seed(47)
    cases, outputs = [], []
    for images, h, w, C, nd, ng in ((3, 24, 37, 3, 9, 6), (2, 16, 16, 2, 12, 4), (4, 20, 30, 4, 15, 8)):
        batch = []
        for _ in range(images):
            gm = torch.rand((ng, h, w), generator=g) > 0.65
            pm = torch.cat([gm[:4].clone(), torch.rand((nd - 4, h, w), generator=g) > 0.65])
            pm[1] &= torch.rand((h, w), generator=g) > 0.2
            pm[2] = gm[0]
            gc = torch.randint(0, C, (ng,), generator=g)
            pc = torch.cat([gc[:4], torch.randint(0, C, (nd - 4,), generator=g)])
            pc[2] = gc[0]
            scores = torch.tensor([0.1, 0.5, 0.9], dtype=torch.float64)[torch.randint(3, (nd,), generator=g)]
            crowd = torch.rand(ng, generator=g) < 0.3
            areas = torch.tensor([100.0, 1024.0, 1025.0, 9216.0, 9217.0],
                                 dtype=torch.float64)[torch.randint(5, (ng,), generator=g)]
            batch.append(dict(pm=pm, pc=pc, scores=scores, gm=gm, gc=gc, crowd=crowd, areas=areas))
        ev = pe.InstanceEvaluator(C, device="cpu")
        for item in batch:  # one update per image, accumulated
            ev.update(pe.InstanceBatch([item["pm"]], [item["pc"]], [item["scores"]]),
                      pe.InstanceBatch([item["gm"]], [item["gc"]], crowd=[item["crowd"]], areas=[item["areas"]]))
        cases.append(dict(images=batch, C=C))
        outputs.append(ev.compute())
    # Known answers: top-100 cap across categories (test_instance.py:179-197).
    masks = torch.ones((106, 1, 1), dtype=torch.bool)
    labels = torch.zeros(106, dtype=torch.int64)
    labels[-1] = 1
    ev = pe.InstanceEvaluator(2, device="cpu")
    ev.update(pe.InstanceBatch([masks], [labels], [torch.ones(106, dtype=torch.float64)]),
              pe.InstanceBatch([masks], [labels]))
    cases.append(dict(images=[dict(pm=masks, pc=labels, scores=torch.ones(106, dtype=torch.float64), gm=masks,
                                   gc=labels, crowd=torch.zeros(106, dtype=torch.bool),
                                   areas=torch.ones(106, dtype=torch.float64))], C=2))
    outputs.append(ev.compute())
    save("instance", cases, outputs)


def combined_cases(pe):
    """SegmentationEvaluator on CPU (combined.py:18-167), fixture of the reference tests."""
    generator = torch.Generator().manual_seed(91)
    maps = torch.randint(0, 6, (2, 13, 35), generator=generator).int()
    classes = torch.tensor([[-1, 0, 1, 0, 2, -1], [-1, 1, 0, 2, 0, 1]], dtype=torch.int32)
    maps[0][maps[0] == 5] = 0
    crowd = torch.tensor([[False, False, True, False, False, False],
                          [False, False, False, False, True, False]])
    pred_maps = maps.clone()
    pred_maps[:, :3] = 0
    masks = [torch.rand((8, 13, 35), generator=generator) > 0.7 for _ in range(2)]
    for b in range(2):
        masks[b][:3] = maps[b][None] == torch.tensor([1, 2, 3])[:, None, None]
    masks[0][3] = True
    labels = [torch.tensor([0, 1, 0, 0, 1, 0, 1, 0]), torch.tensor([1, 0, 0, 1, 0, 1, 0, 1])]
    scores = [torch.tensor([0.9, 0.9, 0.8, 0.5, 0.5, 0.5, 0.1, 0.1], dtype=torch.float64) for _ in range(2)]
    areas = torch.tensor([[0.0, 1024.0, 1025.0, 9216.0, 9217.0, 0.0],
                          [0.0, 100.0, 1024.0, 200.0, 9217.0, 9216.0]], dtype=torch.float64)
    joint = pe.SegmentationEvaluator(3, isthing=[True, True, False], device="cpu")
    for annotation_areas in (None, areas):
        joint.update(pe.PanopticBatch(pred_maps, classes.clone()), pe.InstanceBatch(masks, labels, scores),
                     pe.PanopticBatch(maps, classes, crowd), instance_areas=annotation_areas)
    save("combined", dict(maps=maps, classes=classes, crowd=crowd, pred_maps=pred_maps, masks=masks,
                          labels=labels, scores=scores, areas=areas), joint.compute())


def prefix_cases(pe):
    """segmentation_prefixes on CPU (prefix.py:12-122)."""
    g = torch.Generator().manual_seed(123)
    cases, outputs = [], []
    for gs, n, thresholds in ((3, 0, (.5, .75)), (9, 17, (.5,) * 5), (12, 9, (.5, .75, .95)), (20, 30, (.3, .5))):
        maps = torch.randint(gs, (1, 19, 23), generator=g).int()
        maps.flatten()[:gs] = torch.arange(gs).int()
        labels = (torch.arange(gs) % 3).int()[None]
        labels[:, 0] = -1
        crowd = torch.rand((1, gs), generator=g) < .3
        crowd[:, 0] = False
        slots = torch.randint(1, gs, (n,), generator=g)
        masks = maps[0][None] == slots[:, None, None]
        if n:
            masks |= torch.rand(masks.shape, generator=g) < .05
        classes = labels[0, slots]
        checkpoints = None if n in (9, 30) else ([0, n] if n else [0])
        result = pe.segmentation_prefixes(pe.InstanceBatch([masks], [classes]),
                                          pe.PanopticBatch(maps, labels, crowd), 3,
                                          isthing=[True, False, True], iou_thresholds=thresholds,
                                          checkpoints=checkpoints)
        cases.append(dict(maps=maps, labels=labels, crowd=crowd, masks=masks, classes=classes,
                          thresholds=torch.tensor(thresholds, dtype=torch.float64),
                          checkpoints=None if checkpoints is None else torch.tensor(checkpoints)))
        outputs.append(result)
    save("prefix", cases, outputs)


def main():
    parser = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    parser.add_argument("--reference", required=True, help="path of a panoptic-evaluator checkout")
    args = parser.parse_args()
    sys.dont_write_bytecode = True
    sys.path.insert(0, args.reference)
    import panoptic_evaluator as pe  # the reference package, CPU path
    torch.set_num_threads(1)
    panoptic_cases(pe)
    original_id_cases(pe)
    reward_cases(pe)
    matcher_cases()
    instance_cases(pe)
    combined_cases(pe)
    prefix_cases(pe)
    for path in sorted(HERE.glob("*.npz")):
        print(f"{path.name}: {path.stat().st_size} bytes")


if __name__ == "__main__":
    main()
