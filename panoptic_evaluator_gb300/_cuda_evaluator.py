"""Drop-in module for the reference's ``panoptic_evaluator._cuda_evaluator``.

It exposes the reference extension's op names and signatures
(panoptic_evaluator/csrc/bindings.cpp:28-57) on top of the pe_gb300 C ABI, so
the reference's own Python layer can import this module in its place. Tensor
checks raise ``RuntimeError`` like the reference's ``TORCH_CHECK``; ops that
allocate in the reference allocate their outputs here with torch, then call
the C ABI on the current stream.
"""

from __future__ import annotations

import torch

from . import _native as N


def _require(condition, message):
    if not condition:
        raise RuntimeError(message)


def _check(tensor, reference, dtype, name="tensor"):
    _require(tensor.device == reference.device and tensor.is_contiguous() and tensor.dtype == dtype,
             f"incorrect {name} device, layout or dtype")


def _lookup(ids, slots, classes, reference):
    _require((ids is None) == (slots is None), "lookup IDs and slots must be supplied together")
    if ids is None:
        return None, None
    _check(ids, reference, torch.int64, "lookup IDs")
    _check(slots, reference, torch.int32, "lookup slots")
    _require(ids.shape == classes.shape and slots.shape == classes.shape, "incorrect lookup shape")
    return ids, slots


def update(gt, pred, gc, pc, crowd, pairs, areas, matched, tp, fp, fn, iou_sum, confusion,
           gt_ids=None, gt_slots=None, pred_ids=None, pred_slots=None, error=None, validate=True, reward=False):
    """Count intersections, validate and accumulate (histogram_kernel.cu:257-341)."""
    _require(gt.is_cuda and gt.dim() == 3, "gt must be CUDA B x H x W")
    for t in (gt, pred):
        _require(t.device == gt.device and t.is_contiguous() and t.dtype in (torch.int32, torch.int64),
                 "maps must be contiguous int32 or int64 on the same CUDA device")
    for t in (gc, pc, matched, error):
        _check(t, gt, torch.int32)
    for t in (pairs, areas, tp, fp, fn, confusion):
        _check(t, gt, torch.int64)
    _check(crowd, gt, torch.bool, "crowd")
    _check(iou_sum, gt, torch.float64, "iou_sum")
    _require(pred.shape == gt.shape and gc.dim() == 2 and pc.dim() == 2 and gc.shape[0] == gt.shape[0]
             and pc.shape[0] == gt.shape[0] and crowd.shape == gc.shape, "incorrect input shapes")
    B, G, P = gt.shape[0], gc.shape[1], pc.shape[1]
    C = tp.shape[1] if reward else tp.numel()
    _require(0 < C < 2**31 - 1 and 0 < G < 2**31 - 1 and 0 < P < 2**31 - 1, "invalid capacities")
    _require(tuple(pairs.shape) == (B, G, P) and tuple(areas.shape) == (B, G + P) and matched.shape == gc.shape
             and error.numel() == 1, "incorrect scratch shapes")
    _require((tp.dim() == 2 and tp.shape[0] == B) if reward else tp.dim() == 1, "incorrect state shapes")
    _require(fp.shape == tp.shape and fn.shape == tp.shape and iou_sum.shape == tp.shape
             and (reward or tuple(confusion.shape) == (C, C + 1)), "incorrect state shapes")
    gt_ids, gt_slots = _lookup(gt_ids, gt_slots, gc, gt)
    pred_ids, pred_slots = _lookup(pred_ids, pred_slots, pc, gt)
    with torch.cuda.device(gt.device):
        return N.call("pe_update", N.ptr(gt), int(gt.dtype == torch.int64), N.ptr(pred),
                      int(pred.dtype == torch.int64), B, gt.shape[1] * gt.shape[2], N.ptr(gc), N.ptr(pc),
                      N.ptr(crowd), G, P, C, N.ptr(pairs), N.ptr(areas), N.ptr(matched), N.ptr(tp), N.ptr(fp),
                      N.ptr(fn), N.ptr(iou_sum), None if reward else N.ptr(confusion), N.ptr(gt_ids),
                      N.ptr(gt_slots), N.ptr(pred_ids), N.ptr(pred_slots), N.ptr(error), int(bool(validate)),
                      int(bool(reward)), N.stream_handle())


def _compute_rows(tp, fp, fn, sums, confusion, things, K, C):
    """pe_compute over K rows; every output is a view of one allocation (8-byte words)."""
    sizes = [K * 4 * C, K * 9, K * 3, K, K * C, K * C, K * C, K * C, K * C * (C + 1)]
    flat = torch.empty(sum(sizes), dtype=torch.int64, device=tp.device)
    values, summaries, counts, miou, c_tp, c_fp, c_fn, c_sums, c_conf = flat.split(sizes)
    values = values.view(torch.float64).view(K, 4, C)
    summaries = summaries.view(torch.float64).view(K, 3, 3)
    counts = counts.view(K, 3)
    miou = miou.view(torch.float64)
    copies = [c_tp.view(tp.shape), c_fp.view(fp.shape), c_fn.view(fn.shape), c_sums.view(torch.float64).view(sums.shape),
              c_conf.view(confusion.shape)]
    with N.on_device(tp.device):
        N.call("pe_compute", tp.data_ptr(), fp.data_ptr(), fn.data_ptr(), sums.data_ptr(), confusion.data_ptr(),
               things.data_ptr(), K, C, values.data_ptr(), summaries.data_ptr(), counts.data_ptr(), miou.data_ptr(),
               *[c.data_ptr() for c in copies], N.stream_handle(tp.device))
    return values, summaries, counts, miou, copies


def compute_one(tp, fp, fn, sums, confusion, things, C):
    """pe_compute over one row, its outputs laid out for PanopticEvaluator.compute's result dict.

    Two allocations (FP64: per-class pq, sq, rq, IoU rows, the nine group
    summaries, mIoU, the IoU-sum snapshot; int64: the confusion snapshot, the
    tp / fp / fn snapshots, the three group counts), each split once, so that
    the result costs a handful of tensor views (the host time of this call is
    most of a small evaluation step). Returns (per-class rows [4 tensors of
    C], summaries [9 scalars], counts [3 scalars], miou scalar, [tp, fp, fn,
    sums, confusion] snapshots).
    """
    f64 = torch.empty(5 * C + 10, dtype=torch.float64, device=tp.device)
    i64 = torch.empty(3 + 3 * C + C * (C + 1), dtype=torch.int64, device=tp.device)
    pq, sq, rq, iou, summaries, miou, c_sums = f64.split([C, C, C, C, 9, 1, C])
    # The confusion snapshot first: 16-byte aligned, so the kernel copies it in 16-byte words.
    c_conf, c_tp, c_fp, c_fn, counts = i64.split([C * (C + 1), C, C, C, 3])
    base, ints = f64.data_ptr(), i64.data_ptr()
    tail = ints + 8 * C * (C + 1)
    with N.on_device(tp.device):
        N.call("pe_compute", tp.data_ptr(), fp.data_ptr(), fn.data_ptr(), sums.data_ptr(), confusion.data_ptr(),
               things.data_ptr(), 1, C, base, base + 8 * 4 * C, tail + 8 * 3 * C, base + 8 * (4 * C + 9), tail,
               tail + 8 * C, tail + 8 * 2 * C, base + 8 * (4 * C + 10), ints, N.stream_handle(tp.device))
    return ((pq, sq, rq, iou), summaries.unbind(0), counts.unbind(0), miou.view(()),
            [c_tp, c_fp, c_fn, c_sums, c_conf.view(C, C + 1)])


def compute(tp, fp, fn, sums, confusion, things):
    """Summaries and independent snapshots (compute_kernel.cu:66-95)."""
    _require(tp.is_cuda and tp.dim() == 1 and 0 < tp.numel() < 2**31 - 1, "tp must be nonempty CUDA category counts")
    for t in (tp, fp, fn, sums, confusion, things):
        _require(t.device == tp.device and t.is_contiguous(), "incorrect device or layout")
    for t in (tp, fp, fn, confusion):
        _require(t.dtype == torch.int64, "counts must be int64")
    C = tp.numel()
    _require(fp.shape == tp.shape and fn.shape == tp.shape and sums.shape == tp.shape and things.shape == tp.shape
             and sums.dtype == torch.float64 and things.dtype == torch.bool
             and tuple(confusion.shape) == (C, C + 1), "incorrect state shapes or dtypes")
    values, summaries, counts, miou, copies = _compute_rows(tp, fp, fn, sums, confusion, things, 1, C)
    return [values[0], summaries[0], counts[0], miou[0], *copies]


def compute_prefix(tp, fp, fn, sums, confusion, things):
    """K independent rows (compute_kernel.cu:98-118)."""
    K, C = tp.shape
    values, summaries, counts, miou, copies = _compute_rows(tp, fp, fn, sums, confusion, things, K, C)
    return [values, summaries, counts, miou, *copies]


def pack(maps, ids, slots):
    """Original IDs -> compact slots (histogram_kernel.cu:343-366)."""
    _require(maps.is_cuda and maps.dim() == 3 and maps.is_contiguous() and maps.dtype in (torch.int32, torch.int64),
             "maps must be contiguous CUDA int32 or int64 B x H x W")
    _check(ids, maps, torch.int64, "lookup IDs")
    _check(slots, maps, torch.int32, "lookup slots")
    _require(ids.dim() == 2 and slots.shape == ids.shape and ids.shape[0] == maps.shape[0]
             and 0 < ids.shape[1] < 2**31 - 1, "incorrect lookup shapes")
    output = torch.empty(maps.shape, dtype=torch.int32, device=maps.device)
    error = torch.zeros(1, dtype=torch.int32, device=maps.device)
    with torch.cuda.device(maps.device):
        N.call("pe_pack", N.ptr(maps), int(maps.dtype == torch.int64), maps.shape[0], maps.shape[1] * maps.shape[2],
               N.ptr(ids), N.ptr(slots), ids.shape[1], N.ptr(output), N.ptr(error), N.stream_handle())
    return [output, error]


def _instance_check(x, reference, dtype):
    _require(x.is_cuda and x.device == reference.device and x.is_contiguous() and x.dtype == dtype,
             "invalid instance tensor device, layout or dtype")


def _instance_metadata(reference, pc, gc, pa, ga, crowd, areas, D, G):
    for t in (pc, gc):
        _instance_check(t, reference, torch.int32)
    for t in (pa, ga, areas):
        _instance_check(t, reference, torch.float64)
    _instance_check(crowd, reference, torch.bool)
    _require(D <= 2**31 - 1 and G <= 2**31 - 1 and D * G <= 2**31 - 1, "too many instance pairs")
    for t in (pc, pa):
        _require(t.dim() == 1 and t.numel() == D, "prediction metadata shape mismatch")
    for t in (gc, ga, crowd, areas):
        _require(t.dim() == 1 and t.numel() == G, "target metadata shape mismatch")


def _match(pairs, pc, gc, pa, ga, crowd, areas, C):
    D, G = pairs.shape
    device = pairs.device
    flags = torch.empty((40, D), dtype=torch.int8, device=device)
    ranks = torch.empty(D, dtype=torch.int32, device=device)
    counts = torch.empty((C, 4), dtype=torch.int64, device=device)
    if D == 0:
        flags.fill_(-1)
    with torch.cuda.device(device):
        N.call("pe_instance_match", N.ptr(pairs), D, G, N.ptr(pc), N.ptr(gc), N.ptr(pa), N.ptr(ga), N.ptr(crowd),
               N.ptr(areas), C, N.ptr(flags), N.ptr(ranks), N.ptr(counts), N.stream_handle())
    return [flags, ranks, counts]


def instance_update(pm, gm, pc, gc, pa, ga, crowd, areas, C):
    """Mask IoU and COCO greedy matching (instance_kernel.cu:282-309)."""
    _require(pm.is_cuda and pm.dim() == 3 and gm.dim() == 3 and 0 < C <= (2**31 - 1) // 120,
             "invalid instance masks or category count")
    _instance_check(pm, pm, torch.bool)
    _instance_check(gm, pm, torch.bool)
    _require(pm.shape[1:] == gm.shape[1:] and pm.shape[1] > 0 and pm.shape[2] > 0,
             "instance mask dimensions must match")
    D, G = pm.shape[0], gm.shape[0]
    _instance_metadata(pm, pc, gc, pa, ga, crowd, areas, D, G)
    inter = torch.zeros((D, G), dtype=torch.int64, device=pm.device)
    with torch.cuda.device(pm.device):
        N.call("pe_mask_overlap", N.ptr(pm), D, N.ptr(gm), G, pm.shape[1] * pm.shape[2], N.ptr(pc), N.ptr(gc),
               N.ptr(inter), N.stream_handle())
    return _match(inter, pc, gc, pa, ga, crowd, areas, C)


def instance_match_histogram(pairs, pc, gc, pa, ga, crowd, areas, C):
    """COCO matching from shared target intersections (instance_kernel.cu:365-381)."""
    _require(pairs.is_cuda and pairs.dim() == 2 and 0 < C <= (2**31 - 1) // 120,
             "invalid shared instance intersections or category count")
    _instance_check(pairs, pairs, torch.int64)
    D, G = pairs.shape
    _instance_metadata(pairs, pc, gc, pa, ga, crowd, areas, D, G)
    return _match(pairs, pc, gc, pa, ga, crowd, areas, C)


def instance_histogram(masks, target, order, S):
    """Detection x target-slot pixel counts in score order (instance_kernel.cu:335-363)."""
    _require(masks.is_cuda and masks.dim() == 3 and target.dim() == 2 and 0 < S < 2**31 - 1,
             "invalid shared ground-truth inputs")
    _instance_check(masks, masks, torch.bool)
    _instance_check(target, masks, torch.int32)
    _instance_check(order, masks, torch.int64)
    _require(target.shape[0] == masks.shape[1] and target.shape[1] == masks.shape[2] and target.numel() > 0
             and order.dim() == 1 and order.numel() == masks.shape[0],
             "shared target and detection dimensions must match")
    D = masks.shape[0]
    pairs = torch.zeros((D, S), dtype=torch.int64, device=masks.device)
    with torch.cuda.device(masks.device):
        N.call("pe_instance_histogram", N.ptr(masks), D, target.numel(), N.ptr(target), N.ptr(order), S,
               N.ptr(pairs), N.stream_handle())
    return pairs


def accumulate_workspace(n, C, device):
    bytes_ = N.size("pe_instance_accumulate_workspace", n, C)
    return torch.empty(bytes_, dtype=torch.uint8, device=device)


def instance_compute(classes, ranks, flags, counts):
    """AP/AR accumulation of records in global score order (instance_kernel.cu:311-333)."""
    _require(classes.is_cuda, "instance accumulation requires CUDA")
    _instance_check(classes, classes, torch.int32)
    _instance_check(ranks, classes, torch.int32)
    _instance_check(flags, classes, torch.int8)
    _instance_check(counts, classes, torch.int64)
    _require(classes.dim() == 1 and ranks.shape == classes.shape and flags.dim() == 2 and flags.shape[0] == 40
             and flags.shape[1] == classes.numel() and counts.dim() == 2 and counts.shape[1] == 4
             and 0 < counts.shape[0] <= (2**31 - 1) // 120, "invalid instance state shapes")
    C, n = counts.shape[0], classes.numel()
    precision = torch.empty((10, 101, C, 4, 3), dtype=torch.float64, device=classes.device)
    recall = torch.empty((10, C, 4, 3), dtype=torch.float64, device=classes.device)
    workspace = accumulate_workspace(n, C, classes.device)
    with torch.cuda.device(classes.device):
        N.call("pe_instance_accumulate", N.ptr(classes), N.ptr(ranks), N.ptr(flags), n, 1, None, n, N.ptr(counts), C,
               N.ptr(workspace), workspace.numel(), N.ptr(precision), N.ptr(recall), None, N.stream_handle())
    return [precision, recall]


def prefix(gt, masks, pc, gc, crowd, things, thresholds, points, validate):
    """Fused generation-prefix evaluation of one image (prefix_kernel.cu:142-199).

    Returns the reference's 14 result tensors plus the error word: per-checkpoint
    values, summaries, counts, miou, tp, fp, fn, sums, confusion, then instance
    tp, fp, fn, precision, recall.
    """
    from . import prefix as _prefix
    _require(gt.is_cuda, "prefix inputs must be CUDA tensors")
    for t in (gt, masks, pc, gc, crowd, things, thresholds):
        _require(t.device == gt.device and t.is_contiguous(), "incorrect device or layout")
    _require(gt.dtype == torch.int32 and masks.dtype == torch.bool and pc.dtype == torch.int32
             and gc.dtype == torch.int32 and crowd.dtype == torch.bool and things.dtype == torch.bool
             and thresholds.dtype == torch.float64, "incorrect prefix input dtypes")
    _require(gt.dim() == 2 and masks.dim() == 3 and pc.dim() == 1 and gc.dim() == 1 and crowd.shape == gc.shape
             and things.dim() == 1 and thresholds.dim() == 1 and masks.shape[0] == pc.numel()
             and masks.shape[1:] == gt.shape, "incorrect prefix input shapes")
    n = pc.numel()
    last = -1
    for q in points:
        _require(last < q <= n, "invalid checkpoints")
        last = q
    out, _, code, _ = _prefix.run_prefixes(gt[None], gc[None], crowd[None], [masks], [pc], things.numel(), things,
                                           tuple(thresholds.tolist()), [list(points)], validate)
    error = torch.tensor(code, dtype=torch.int32, device=gt.device)
    return [out[k] for k in ("values", "summaries", "counts", "miou", "tp", "fp", "fn", "sums", "confusion",
                             "itp", "ifp", "ifn", "precision", "recall")] + [error]
