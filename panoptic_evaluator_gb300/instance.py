"""COCO mask AP/AR on the GPU (same API as the reference's ``panoptic_evaluator/instance.py``).

``InstanceEvaluator.update`` evaluates a whole batch with a fixed number of
launches: per-image score sort, one mask-overlap pass over all images, area /
validation prep and batched greedy matching, all on the current stream. Only
records (score, class, rank, 40 match flags per detection) stay on the device
between updates; ``compute`` sorts them by score per class and accumulates
101-point precision/recall in the ``pe_instance_accumulate`` kernel.
"""

from __future__ import annotations

from dataclasses import dataclass
from typing import Sequence

import numpy as np
import torch

from . import _native as N
from ._batch import (CHAINS, CHUNK_BEGIN, D, DET_BEGIN, DPAIR_BEGIN, FLAGS, G, INST_CHUNK, MASK_STRIDE, MASKS, PIXELS,
                     SLOT_BEGIN, TARGET, DescTable, RecordStore, Scratch, aligned, contract_blocks, upload)

# Mask-vs-mask counts: "tensor" runs the tcgen05 contraction (pe_inst_contract),
# "popcount" the bit-packed AND + popcount kernel (pe_inst_overlap). Both are exact.
CONTRACTION = "tensor"

SUMMARY_KEYS = ("ap", "ap50", "ap75", "ap_small", "ar_small", "ap_medium", "ar_medium", "ap_large", "ar_large",
                "ar1", "ar10", "ar100")
_INSTANCE_ERRORS = (
    (32, "scores must be finite; areas must be nonnegative"),
    (64, "areas must be finite; areas must be nonnegative"),
    (8, "classes must be valid category indices"),
    (16, "each instance mask must have pixels"),
)


@dataclass(frozen=True)
class InstanceBatch:
    """One N x H x W bool tensor per image, with N category indices (instance.py:13-26).

    Predictions need floating point scores; targets accept crowd flags and
    annotation areas. Masks may overlap; empty images use N = 0.
    """

    masks: Sequence[torch.Tensor]
    classes: Sequence[torch.Tensor]
    scores: Sequence[torch.Tensor] | None = None
    crowd: Sequence[torch.Tensor] | None = None
    areas: Sequence[torch.Tensor] | None = None


def raise_instance_error(code: int, messages=_INSTANCE_ERRORS):
    for bit, message in messages:
        if code & bit:
            raise ValueError(message)
    if code:
        raise ValueError(f"invalid instance input (code {code})")


def check_instance_batch(batch: InstanceBatch, device, *, prediction: bool):
    """Structural checks of the reference's _prepare (instance.py:78-126); value checks run on the GPU.

    Each tensor's attributes are read once; the per-image conditions are then
    checked over whole lists, and the failing image is located only to raise
    the reference's error for it.
    """
    count = len(batch.masks)
    for field in (batch.classes, batch.scores, batch.crowd, batch.areas):
        if field is not None and len(field) != count:
            raise ValueError("all fields must contain one tensor per image")
    if prediction and batch.scores is None:
        raise ValueError("predictions require scores")
    shapes = [m.shape for m in batch.masks]
    if any(len(s) != 3 or s[1] <= 0 or s[2] <= 0 for s in shapes) or \
            any(m.dtype != torch.bool for m in batch.masks):
        raise ValueError("masks must be bool N x H x W with positive image dimensions")
    lengths = [(s[0],) for s in shapes]
    if [c.shape for c in batch.classes] != lengths or \
            any(c.dtype != torch.int32 and c.dtype != torch.int64 for c in batch.classes):
        raise ValueError("classes must be int32/int64 N tensors")
    for name in ("scores", "crowd", "areas"):
        field = getattr(batch, name)
        if field is None:
            continue
        if [v.shape for v in field] != lengths or any(v.device != device for v in field):
            raise ValueError(f"{name} must have shape N and share evaluator device")
        if name == "crowd":
            if any(v.dtype != torch.bool for v in field):
                raise ValueError("crowd must be bool")
        elif not all(v.is_floating_point() for v in field):
            raise ValueError(f"{name} must be floating point")
    if any(m.device != device for m in batch.masks) or any(c.device != device for c in batch.classes):
        raise ValueError("inputs must share evaluator device")


def _flat(tensors, dtype, device, count):
    """One flat tensor of `dtype` from per-image 1-D tensors (one concatenation, then at most one conversion)."""
    if count == 0:
        return torch.empty(0, dtype=dtype, device=device)
    return torch.cat(list(tensors)).to(dtype)


def summarize(precision, recall, summary):
    """Result dict of the reference's _summarize (instance.py:236-248)."""
    result = {key: summary[i] for i, key in enumerate(SUMMARY_KEYS)}
    result.update(precision=precision, recall=recall)
    return result


class InstanceEvaluator:
    """COCO mask AP/AR with GPU intersections, matching and accumulation (instance.py:46-227)."""

    def __init__(self, num_classes: int, *, device: str | torch.device = "cuda", validate: bool = True):
        if not isinstance(num_classes, int) or isinstance(num_classes, bool) or num_classes <= 0:
            raise ValueError("num_classes must be a positive integer")
        self.num_classes = num_classes
        self.device = torch.device(device)
        if self.device.type != "cuda":
            raise ValueError("pe_gb300 evaluates on CUDA devices only")
        if self.device.index is None:
            self.device = torch.device("cuda", torch.cuda.current_device())
        self.validate = validate
        self._scratch = Scratch(self.device)
        self._store = RecordStore(self.device)
        self.reset()

    def reset(self):
        self._store.reset()
        self._counts = torch.zeros((self.num_classes, 4), dtype=torch.int64, device=self.device)

    @property
    def num_records(self):
        return self._store.n

    def state_dict(self) -> dict:
        """Positives per (class, area range) and the records (copies), in update order."""
        store, n = self._store, self._store.n
        return {"counts": self._counts.clone(), "records.scores": store.scores[:n].clone(),
                "records.classes": store.classes[:n].clone(), "records.ranks": store.ranks[:n].clone(),
                "records.flags": store.flags[:n].clone()}

    def load_state_dict(self, state: dict):
        """Replace positives and records (for example with replicas merged by ``distributed``)."""
        counts = state["counts"]
        if counts.shape != self._counts.shape:
            raise ValueError(f"counts: expected shape {tuple(self._counts.shape)}, got {tuple(counts.shape)}")
        n = int(state["records.scores"].shape[0])
        if any(state[f"records.{k}"].shape[0] != n for k in ("classes", "ranks", "flags")) or \
                state["records.flags"].shape[1:] != (CHAINS,):
            raise ValueError("records must hold one score, class, rank and 40 flags per detection")
        store = self._store
        store.reset()
        store.reserve(n)
        dev = self.device
        store.scores[:n].copy_(state["records.scores"].to(dev, torch.float64))
        store.classes[:n].copy_(state["records.classes"].to(dev, torch.int32))
        store.ranks[:n].copy_(state["records.ranks"].to(dev, torch.int32))
        store.flags[:n].copy_(state["records.flags"].to(dev, torch.int8))
        store.n = n
        self._counts.copy_(counts.to(dev, torch.int64))
        return self

    @torch.no_grad()
    def update(self, prediction: InstanceBatch, target: InstanceBatch):
        check_instance_batch(prediction, self.device, prediction=True)
        check_instance_batch(target, self.device, prediction=False)
        if len(prediction.masks) != len(target.masks) or any(
                p.shape[1:] != g.shape[1:] for p, g in zip(prediction.masks, target.masks)):
            raise ValueError("prediction and target must have matching image counts and dimensions")
        B = len(prediction.masks)
        if B == 0:
            return self
        dev, S = self.device, self._scratch
        dets = np.array([m.shape[0] for m in prediction.masks], np.int64)
        gts = np.array([m.shape[0] for m in target.masks], np.int64)
        total_d, total_g = int(dets.sum()), int(gts.sum())
        table = DescTable(B)
        d = table.desc
        pixels = np.array([m.shape[1] * m.shape[2] for m in prediction.masks], np.int64)
        # Kernels read mask rows through raw pointers: keep contiguous tensors alive for the call.
        pred_masks = [m.contiguous() for m in prediction.masks]
        gt_masks = [m.contiguous() for m in target.masks]
        d[:, PIXELS] = pixels
        d[:, MASK_STRIDE] = pixels
        d[:, MASKS] = [m.data_ptr() for m in pred_masks]
        d[:, TARGET] = [m.data_ptr() for m in gt_masks]
        d[:, D] = dets
        d[:, G] = gts
        d[:, DET_BEGIN] = np.cumsum(dets) - dets
        d[:, SLOT_BEGIN] = np.cumsum(gts) - gts
        pairs = dets * gts
        d[:, DPAIR_BEGIN] = np.cumsum(pairs) - pairs
        chunks = (pixels + INST_CHUNK - 1) // INST_CHUNK
        d[:, CHUNK_BEGIN] = np.cumsum(chunks) - chunks
        d[:, FLAGS] = [2 * int(aligned(p.data_ptr(), int(n)) and aligned(g.data_ptr(), int(n)))
                       for p, g, n in zip(pred_masks, gt_masks, pixels)]
        table.finish(S, "inst_descs")
        pc = _flat(prediction.classes, torch.int32, dev, total_d)
        scores = _flat(prediction.scores, torch.float64, dev, total_d)
        gc = _flat(target.classes, torch.int32, dev, total_g)
        crowd = (_flat(target.crowd, torch.uint8, dev, total_g) if target.crowd is not None
                 else torch.zeros(total_g, dtype=torch.uint8, device=dev))
        ann = _flat(target.areas, torch.float64, dev, total_g) if target.areas is not None else None
        store = self._store
        store.reserve(total_d)
        out_scores, out_classes, out_ranks, out_flags = store.tail()
        error = S.get("error", 1, torch.int32, zero=True)
        order = S.get("order", total_d, torch.int64)
        ws_bytes = N.size("pe_seg_sort_workspace", total_d)
        ws = S.get("sort_ws", ws_bytes, torch.uint8)
        inter = S.get("inter", int(pairs.sum()), torch.int32)
        pa_count = S.get("pa_count", total_d, torch.int64)
        ga_count = S.get("ga_count", total_g, torch.int64)
        pa = S.get("pa", total_d, torch.float64)
        ga = S.get("ga", total_g, torch.float64)
        ann_out = S.get("ann", total_g, torch.float64)
        stream = N.stream_handle(dev)
        C = self.num_classes
        with torch.cuda.device(dev):
            N.call("pe_seg_sort", N.ptr(table.descs), B, N.ptr(scores), N.ptr(pc), total_d, N.ptr(order),
                   N.ptr(out_scores), N.ptr(out_classes), N.ptr(ws), ws.numel(), stream)
            overlaps(S, table, dets, gts, pixels, chunks, order, out_classes, gc, inter, int(pairs.sum()), pa_count,
                     total_d, ga_count, total_g, error, stream)
            N.call("pe_inst_prepare", N.ptr(table.descs), B, N.ptr(pa_count), N.ptr(ga_count), N.ptr(pa), N.ptr(ga),
                   N.ptr(out_classes), N.ptr(gc), N.ptr(out_scores), N.ptr(ann), N.ptr(ann_out), C,
                   int(self.validate), N.ptr(error), stream)
            N.call("pe_seg_match", N.ptr(inter), N.ptr(table.pair_off), N.ptr(table.d_off), N.ptr(table.g_off), B,
                   N.ptr(out_classes), N.ptr(pa), N.ptr(gc), N.ptr(ga), N.ptr(crowd), N.ptr(ann_out), C,
                   int(max(gts.max(), 1)), N.ptr(out_flags), 1, CHAINS, N.ptr(out_ranks), N.ptr(self._counts),
                   N.ptr(error), stream)
        if self.validate:
            raise_instance_error(int(error.item()))
        store.n += total_d
        return self

    @torch.no_grad()
    def compute(self):
        """COCO AP/AR summaries plus full precision / recall arrays."""
        return accumulate_records(self._store, self._counts, self.num_classes, self._scratch)


def overlaps(scratch, table, dets, gts, pixels, chunks, order, pc, gc, inter, inter_len, pa, pa_len, ga, ga_len, error,
             stream, method=None):
    """Detection x target intersections (u32, rows in score order) and both u64 mask areas."""
    if (method or CONTRACTION) == "tensor":
        blocks, total, bounds = contract_blocks(dets, gts, pixels, ctas=N.sm_count(scratch.device))
        host = np.concatenate((blocks.reshape(-1), bounds))
        buf = upload(host, scratch.get("contract_blocks", host.size, torch.int64))
        N.call("pe_inst_contract", N.ptr(table.descs), N.ptr(buf), len(blocks), total, N.ptr(buf[blocks.size:]),
               len(bounds) - 1, N.ptr(order), N.ptr(inter), inter_len, N.ptr(pa), pa_len, N.ptr(ga), ga_len,
               N.ptr(error), stream)
    else:
        N.call("pe_inst_overlap", N.ptr(table.descs), len(dets), int(chunks.sum()), int((dets + gts).max()),
               N.ptr(order), N.ptr(pc), N.ptr(gc), N.ptr(inter), inter_len, N.ptr(pa), pa_len, N.ptr(ga), ga_len,
               stream)


@torch.no_grad()
def pairwise_intersections(pred_masks, gt_masks, *, method=None):
    """Per image: (intersections [D, G], prediction areas [D], target areas [G]) as int64 CUDA tensors.

    Exact pixel counts of every pair of N x H x W bool masks on the GPU (the
    contraction InstanceEvaluator matches with; the popcount kernel with
    ``method="popcount"``, which counts only same-class pairs and so is not
    offered here).
    """
    if (method or CONTRACTION) != "tensor":
        raise ValueError('pairwise_intersections supports method="tensor" only')
    if len(pred_masks) != len(gt_masks):
        raise ValueError("one prediction and one target mask tensor per image")
    if not pred_masks:
        return []
    dev = pred_masks[0].device
    if dev.type != "cuda":
        raise ValueError("pe_gb300 evaluates on CUDA devices only")
    pm = [m.contiguous() for m in pred_masks]
    gm = [m.contiguous() for m in gt_masks]
    for p, g in zip(pm, gm):
        if p.dtype != torch.bool or g.dtype != torch.bool or p.ndim != 3 or g.ndim != 3 or p.shape[1:] != g.shape[1:] \
                or p.device != dev or g.device != dev:
            raise ValueError("masks must be bool N x H x W tensors of matching image size on one device")
    dets = np.array([m.shape[0] for m in pm], np.int64)
    gts = np.array([m.shape[0] for m in gm], np.int64)
    pixels = np.array([m.shape[1] * m.shape[2] for m in pm], np.int64)
    B = len(pm)
    scratch = Scratch(dev)
    table = DescTable(B)
    d = table.desc
    d[:, PIXELS] = pixels
    d[:, MASK_STRIDE] = pixels
    d[:, MASKS] = [m.data_ptr() for m in pm]
    d[:, TARGET] = [m.data_ptr() for m in gm]
    d[:, D] = dets
    d[:, G] = gts
    d[:, DET_BEGIN] = np.cumsum(dets) - dets
    d[:, SLOT_BEGIN] = np.cumsum(gts) - gts
    pairs = dets * gts
    d[:, DPAIR_BEGIN] = np.cumsum(pairs) - pairs
    table.finish(scratch, "descs")
    order = torch.from_numpy(np.concatenate([np.arange(n) for n in dets]) if dets.sum() else
                             np.zeros(0, np.int64)).to(dev)
    inter = torch.empty(max(int(pairs.sum()), 1), dtype=torch.int32, device=dev)
    pa = torch.empty(max(int(dets.sum()), 1), dtype=torch.int64, device=dev)
    ga = torch.empty(max(int(gts.sum()), 1), dtype=torch.int64, device=dev)
    error = torch.zeros(1, dtype=torch.int32, device=dev)
    with torch.cuda.device(dev):
        overlaps(scratch, table, dets, gts, pixels, None, order, None, None, inter, int(pairs.sum()), pa,
                 int(dets.sum()), ga, int(gts.sum()), error, N.stream_handle(dev), method="tensor")
    if int(error.item()):
        raise RuntimeError(f"mask contraction failed (error bits {int(error.item()):#x})")
    out = []
    for b in range(B):
        p0, d0, g0 = int(d[b, DPAIR_BEGIN]), int(d[b, DET_BEGIN]), int(d[b, SLOT_BEGIN])
        counts = inter[p0: p0 + int(pairs[b])].view(torch.int32).to(torch.int64) & 0xFFFFFFFF
        out.append((counts.reshape(int(dets[b]), int(gts[b])), pa[d0: d0 + int(dets[b])].clone(),
                    ga[g0: g0 + int(gts[b])].clone()))
    return out


def accumulate_records(store: RecordStore, counts, C, scratch: Scratch):
    dev = counts.device
    n = store.n
    precision = torch.empty((10, 101, C, 4, 3), dtype=torch.float64, device=dev)
    recall = torch.empty((10, C, 4, 3), dtype=torch.float64, device=dev)
    summary = torch.empty(12, dtype=torch.float64, device=dev)
    ws = scratch.get("acc_ws", N.size("pe_instance_accumulate_workspace", n, C), torch.uint8)
    stream = N.stream_handle(dev)
    with torch.cuda.device(dev):
        N.call("pe_instance_accumulate", N.ptr(store.classes), N.ptr(store.ranks), N.ptr(store.flags), 1, CHAINS,
               N.ptr(store.scores), n, N.ptr(counts), C, N.ptr(ws), ws.numel(), N.ptr(precision), N.ptr(recall),
               N.ptr(summary), stream)
    return summarize(precision, recall, summary)
