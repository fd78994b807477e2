"""COCO mask AP/AR on the GPU (same API as the reference's ``panoptic_evaluator/instance.py``).

``InstanceEvaluator.update`` evaluates a whole batch with a fixed number of
launches: per-image score sort, one mask-overlap pass over all images, area /
validation prep and batched greedy matching, all on the current stream. Only
records (score, class, rank, 40 match flags per detection) stay on the device
between updates; ``compute`` sorts them by score per class and accumulates
101-point precision/recall in the ``pe_instance_accumulate`` kernel.
"""

from __future__ import annotations

import itertools
from dataclasses import dataclass
from typing import Sequence

import numpy as np
import torch

from . import _native as N
from ._batch import (CHAINS, CHUNK_BEGIN, D, DET_BEGIN, DPAIR_BEGIN, FLAGS, G, INST_CHUNK, MASK_STRIDE, MASKS, PIXELS,
                     SLOT_BEGIN, TARGET, DescTable, RecordStore, Scratch, aligned, contract_blocks)

# Mask-vs-mask counts: "tensor" runs the tcgen05 contraction (pe_inst_contract),
# "popcount" the bit-packed AND + popcount kernel (pe_inst_overlap). Both are exact.
CONTRACTION = "tensor"
# Images whose mask rows start on 16-byte boundaries are loaded into the
# contraction's operand tiles by TMA (tensor maps) instead of being staged and
# re-aligned by the worker warps.
DIRECT_CONTRACTION = True

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


# Error bits from 2^20 up are raised by the mask contraction itself, not by the input: bit 30 a wait
# that timed out (bits 20-25 name its site), bit 28 TMA blocks placed before staged ones.
_KERNEL_BITS = ~((1 << 20) - 1)


def raise_instance_error(code: int, messages=_INSTANCE_ERRORS):
    if code & _KERNEL_BITS:
        raise RuntimeError(f"mask contraction stopped (error bits {code:#x})")
    for bit, message in messages:
        if code & bit:
            raise ValueError(message)
    if code:
        raise ValueError(f"invalid instance input (code {code})")


_INDEX_DTYPES = frozenset((torch.int32, torch.int64))


def check_instance_batch(batch: InstanceBatch, device, *, prediction: bool):
    """Structural checks of the reference's _prepare (instance.py:78-126); value checks run on the GPU.

    Each tensor's attributes are read once, list by list; the per-image
    conditions are then checked over whole lists (dtypes and devices as
    sets) in the reference's order. An image with one fault gets the
    reference's message; with faults of different kinds in several images,
    the first kind in that order is reported (the reference reports the
    first image's). Returns what the update needs of them: the mask shapes
    and, per metadata field present, the dtypes of its tensors.
    """
    count = len(batch.masks)
    for field in (batch.classes, batch.scores, batch.crowd, batch.areas):
        if field is not None and len(field) != count:
            raise ValueError("all fields must contain one tensor per image")
    if prediction and batch.scores is None:
        raise ValueError("predictions require scores")
    masks = batch.masks
    shapes = [m.shape for m in masks]
    if any(len(s) != 3 or s[1] <= 0 or s[2] <= 0 for s in shapes) or {m.dtype for m in masks} - {torch.bool}:
        raise ValueError("masks must be bool N x H x W with positive image dimensions")
    lengths = [(s[0],) for s in shapes]
    class_dtypes = [c.dtype for c in batch.classes]
    if [c.shape for c in batch.classes] != lengths or not set(class_dtypes) <= _INDEX_DTYPES:
        raise ValueError("classes must be int32/int64 N tensors")
    dtypes = {"classes": class_dtypes}
    for name in ("scores", "crowd", "areas"):
        field = getattr(batch, name)
        if field is None:
            continue
        if [v.shape for v in field] != lengths or {v.device for v in field} - {device}:
            raise ValueError(f"{name} must have shape N and share evaluator device")
        kinds = [v.dtype for v in field]
        if name == "crowd":
            if set(kinds) - {torch.bool}:
                raise ValueError("crowd must be bool")
        elif not all(kind.is_floating_point for kind in set(kinds)):
            raise ValueError(f"{name} must be floating point")
        dtypes[name] = kinds
    if {m.device for m in masks} - {device} or {c.device for c in batch.classes} - {device}:
        raise ValueError("inputs must share evaluator device")
    return shapes, dtypes


def shape_table(shapes):
    """int64 [n, 3] array of n three-dimensional shapes (torch.Size objects)."""
    return np.fromiter(itertools.chain.from_iterable(shapes), np.int64, 3 * len(shapes)).reshape(-1, 3)


@dataclass
class ContractPlan:
    """pe_inst_contract's block table, CTA bounds and tensor maps, laid out to travel with the descriptors.

    ``extra`` goes to ``DescTable.finish(bounds=extra)``; the device offsets of
    its parts are then read from ``table.bounds``.
    """
    extra: np.ndarray
    blocks: np.ndarray
    total_chunks: int
    ctas: int
    maps_at: int  # int64 index of the tensor maps in extra, -1 without maps

    def pointers(self, table):
        base = table.bounds.data_ptr() if table.bounds is not None else None
        if base is None or not self.total_chunks:
            return None, None, None
        return base, base + 8 * self.blocks.size, (base + 8 * self.maps_at if self.maps_at >= 0 else None)


def contract_plan(table, dets, gts, pixels, device, direct=None):
    """Block table and CTA bounds of the contraction, plus tensor maps for images with 16-byte rows.

    Call before ``table.finish``: pe_contract_maps marks the images it gives
    maps (descriptor flags bit 2) in the host table, and their blocks are
    placed after the staged images' blocks.
    """
    direct = DIRECT_CONTRACTION if direct is None else direct
    B = table.B
    maps = None
    if direct and B:
        raw = np.zeros(B * 32 + 8, np.int64)  # two 128-byte CUtensorMap per image, on a 64-byte boundary
        maps = raw[(-raw.ctypes.data // 8) % 8:][: B * 32]
        if not N.call("pe_contract_maps", table.desc.ctypes.data, B, maps.ctypes.data):
            maps = None
    tma = (table.desc[:, FLAGS] & 4) != 0 if maps is not None else None
    cost = None
    if tma is not None:
        from . import tuning
        cost = tuning.contract_cost(tuning.contract_bucket(dets, gts, pixels, tma))
    blocks, total, bounds = contract_blocks(dets, gts, pixels, ctas=N.sm_count(device), tma=tma, tma_cost=cost)
    head = np.concatenate((blocks.reshape(-1), bounds))
    if maps is None or not total:
        return ContractPlan(head, blocks, total, len(bounds) - 1, -1)
    # extra starts table.extra_offset() int64 into the upload; the maps start on a 64-byte boundary of it.
    pad = -(table.extra_offset() + head.size) % 8
    extra = np.concatenate((head, np.zeros(pad, np.int64), maps))
    return ContractPlan(extra, blocks, total, len(bounds) - 1, head.size + pad)


def mask_flags(pm_ptr, gm_ptr, pixels):
    """Descriptor flags of mask rows: bit 1 when every row starts on a 16-byte boundary.

    Rows of an image start at base + r x H x W, so this holds for every row
    when both bases and H x W are multiples of 16.
    """
    pm_ptr, gm_ptr, pixels = (np.asarray(x, np.int64) for x in (pm_ptr, gm_ptr, pixels))
    return 2 * ((pm_ptr % 16 == 0) & (gm_ptr % 16 == 0) & (pixels % 16 == 0)).astype(np.int64)


# pe_inst_gather's per-image row: (column, element-size bit, narrow dtype, wide dtype) of each field.
_GATHER = ((0, 1, torch.int32, torch.int64), (1, 2, torch.float32, torch.float64), (2, 4, torch.int32, torch.int64),
           (3, 0, torch.bool, torch.bool), (4, 16, torch.float32, torch.float64))


def gather_rows(prediction: InstanceBatch, target: InstanceBatch, B: int, dtypes=None):
    """pe_inst_gather's rows (field pointers and element sizes per image), or None for torch's path.

    Fields of other dtypes (for example float16 scores) or strided 1-D
    tensors take the concatenation path, which converts them. ``dtypes``:
    the (prediction, target) dtype lists that check_instance_batch returned,
    read here otherwise.
    """
    rows = np.zeros((B, 6), np.int64)
    pred_kinds, target_kinds = dtypes if dtypes is not None else ({}, {})
    fields = ((prediction.classes, pred_kinds.get("classes")), (prediction.scores, pred_kinds.get("scores")),
              (target.classes, target_kinds.get("classes")), (target.crowd, target_kinds.get("crowd")),
              (target.areas, target_kinds.get("areas")))
    for (col, bit, narrow, wide), (tensors, kinds) in zip(_GATHER, fields):
        if tensors is None:
            continue
        if kinds is None:
            kinds = [t.dtype for t in tensors]
        present = set(kinds)
        if present - {narrow, wide} or not all([t.is_contiguous() for t in tensors]):
            return None
        rows[:, col] = [t.data_ptr() for t in tensors]
        if bit and wide in present and wide is not narrow:
            rows[:, 5] |= bit if len(present) == 1 else bit * np.fromiter((k is wide for k in kinds), np.int64, B)
    return rows


def _flat(tensors, dtype, device, count):
    """One flat tensor of `dtype` from per-image 1-D tensors (one concatenation, then at most one conversion)."""
    if count == 0:
        return torch.empty(0, dtype=dtype, device=device)
    return torch.cat(list(tensors)).to(dtype)


def summarize(precision, recall, summary):
    """Result dict of the reference's _summarize (instance.py:236-248)."""
    result = dict(zip(SUMMARY_KEYS, summary.unbind(0)))  # 0-dim views, one call
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
        pred_shapes, pred_kinds = check_instance_batch(prediction, self.device, prediction=True)
        gt_shapes, gt_kinds = check_instance_batch(target, self.device, prediction=False)
        B = len(prediction.masks)
        if len(target.masks) != B:
            raise ValueError("prediction and target must have matching image counts and dimensions")
        if B == 0:
            return self
        shapes, gt_table = shape_table(pred_shapes), shape_table(gt_shapes)
        if (shapes[:, 1:] != gt_table[:, 1:]).any():
            raise ValueError("prediction and target must have matching image counts and dimensions")
        dev, S = self.device, self._scratch
        # Kernels read mask rows through raw pointers: keep contiguous tensors alive for the call.
        pred_masks = [m.contiguous() for m in prediction.masks]
        gt_masks = [m.contiguous() for m in target.masks]
        dets = shapes[:, 0]
        gts = gt_table[:, 0]
        pixels = shapes[:, 1] * shapes[:, 2]
        pm_ptr = np.array([m.data_ptr() for m in pred_masks], np.int64)
        gm_ptr = np.array([m.data_ptr() for m in gt_masks], np.int64)
        total_d, total_g = int(dets.sum()), int(gts.sum())
        table = DescTable(B)
        d = table.desc
        d[:, PIXELS] = pixels
        d[:, MASK_STRIDE] = pixels
        d[:, MASKS] = pm_ptr
        d[:, TARGET] = gm_ptr
        d[:, D] = dets
        d[:, G] = gts
        d[:, DET_BEGIN] = np.cumsum(dets) - dets
        d[:, SLOT_BEGIN] = np.cumsum(gts) - gts
        pairs = dets * gts
        d[:, DPAIR_BEGIN] = np.cumsum(pairs) - pairs
        chunks = (pixels + INST_CHUNK - 1) // INST_CHUNK
        d[:, CHUNK_BEGIN] = np.cumsum(chunks) - chunks
        d[:, FLAGS] = mask_flags(pm_ptr, gm_ptr, pixels)
        # The contraction's block table, CTA bounds and tensor maps, and the per-image field pointers of the
        # metadata gather, travel with the descriptors (one upload).
        tensor = CONTRACTION == "tensor"
        plan = contract_plan(table, dets, gts, pixels, dev) if tensor else None
        rows = gather_rows(prediction, target, B, (pred_kinds, gt_kinds))
        head = plan.extra if tensor else np.zeros(0, np.int64)
        extra = np.concatenate((head, rows.reshape(-1))) if rows is not None else head
        table.finish(S, "inst_descs", bounds=extra if extra.size else None)
        if rows is not None:
            pc = S.get("pc", total_d, torch.int32)
            scores = S.get("scores", total_d, torch.float64)
            gc = S.get("gc", total_g, torch.int32)
            crowd = S.get("crowd", total_g, torch.uint8)
            ann = S.get("ann_in", total_g, torch.float64) if target.areas is not None else None
            with N.on_device(dev):
                N.call("pe_inst_gather", table.descs.data_ptr(), table.bounds.data_ptr() + 8 * head.size, B,
                       pc.data_ptr(), scores.data_ptr(), gc.data_ptr(), crowd.data_ptr(), N.ptr(ann),
                       N.stream_handle(dev))
        else:
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
        inter_len = int(pairs.sum())
        inter = S.get("inter", inter_len, torch.int32)
        pa_count = S.get("pa_count", total_d, torch.int64)
        ga_count = S.get("ga_count", total_g, torch.int64)
        pa = S.get("pa", total_d, torch.float64)
        ga = S.get("ga", total_g, torch.float64)
        ann_out = S.get("ann", total_g, torch.float64)
        class_bits = S.get("class_bits", B * ((self.num_classes + 31) // 32), torch.int32)
        stream = N.stream_handle(dev)
        C = self.num_classes
        descs = table.descs.data_ptr()
        with N.on_device(dev):
            N.call("pe_seg_sort", descs, B, scores.data_ptr(), pc.data_ptr(), total_d, order.data_ptr(),
                   out_scores.data_ptr(), out_classes.data_ptr(), ws.data_ptr(), ws.numel(), stream)
            if tensor:
                contract(table, plan, order, inter, inter_len, pa_count, total_d, ga_count, total_g, error, stream)
            else:
                overlaps(S, table, dets, gts, pixels, chunks, order, out_classes, gc, inter, inter_len, pa_count,
                         total_d, ga_count, total_g, error, stream, method="popcount")
            N.call("pe_inst_prepare", descs, B, pa_count.data_ptr(), ga_count.data_ptr(), pa.data_ptr(),
                   ga.data_ptr(), out_classes.data_ptr(), gc.data_ptr(), out_scores.data_ptr(), N.ptr(ann),
                   ann_out.data_ptr(), C, int(self.validate), class_bits.data_ptr(), error.data_ptr(), stream)
            N.call("pe_seg_match", inter.data_ptr(), table.pair_off.data_ptr(), table.d_off.data_ptr(),
                   table.g_off.data_ptr(), B, out_classes.data_ptr(), pa.data_ptr(), gc.data_ptr(), ga.data_ptr(),
                   crowd.data_ptr(), ann_out.data_ptr(), C, int(max(gts.max(), 1)), out_flags.data_ptr(), 1, CHAINS,
                   out_ranks.data_ptr(), self._counts.data_ptr(), error.data_ptr(), class_bits.data_ptr(), stream)
        if self.validate:
            raise_instance_error(int(error.item()))
        store.n += total_d
        return self

    @torch.no_grad()
    def compute(self):
        """COCO AP/AR summaries plus full precision / recall arrays."""
        return accumulate_records(self._store, self._counts, self.num_classes, self._scratch)


def contract(table, plan, order, inter, inter_len, pa, pa_len, ga, ga_len, error, stream):
    """pe_inst_contract over a finished table whose upload carried ``plan.extra``."""
    blocks, bounds, maps = plan.pointers(table)
    N.call("pe_inst_contract", table.descs.data_ptr(), blocks, len(plan.blocks), plan.total_chunks, bounds, plan.ctas,
           order.data_ptr(), inter.data_ptr(), inter_len, pa.data_ptr(), pa_len, ga.data_ptr(), ga_len, maps,
           error.data_ptr(), stream)


def overlaps(scratch, table, dets, gts, pixels, chunks, order, pc, gc, inter, inter_len, pa, pa_len, ga, ga_len, error,
             stream, method=None, plan=None):
    """Detection x target intersections (u32, rows in score order) and both u64 mask areas."""
    if (method or CONTRACTION) == "tensor":
        contract(table, plan, order, inter, inter_len, pa, pa_len, ga, ga_len, error, stream)
    else:
        N.call("pe_inst_overlap", N.ptr(table.descs), len(dets), int(chunks.sum()), int((dets + gts).max()),
               N.ptr(order), N.ptr(pc), N.ptr(gc), N.ptr(inter), inter_len, N.ptr(pa), pa_len, N.ptr(ga), ga_len,
               stream)


@torch.no_grad()
def pairwise_intersections(pred_masks, gt_masks, *, method=None, direct=None):
    """Per image: (intersections [D, G], prediction areas [D], target areas [G]) as int64 CUDA tensors.

    Exact pixel counts of every pair of N x H x W bool masks on the GPU (the
    contraction InstanceEvaluator matches with; the popcount kernel with
    ``method="popcount"``, which counts only same-class pairs and so is not
    offered here). ``direct=False`` stages every image through the worker warps,
    also those whose rows TMA could load into the operand tiles directly.
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
    d[:, FLAGS] = mask_flags(d[:, MASKS], d[:, TARGET], pixels)
    plan = contract_plan(table, dets, gts, pixels, dev, direct)
    table.finish(scratch, "descs", bounds=plan.extra)
    order = torch.from_numpy(np.concatenate([np.arange(n) for n in dets]) if dets.sum() else
                             np.zeros(0, np.int64)).to(dev)
    inter = torch.empty(max(int(pairs.sum()), 1), dtype=torch.int32, device=dev)
    pa = torch.empty(max(int(dets.sum()), 1), dtype=torch.int64, device=dev)
    ga = torch.empty(max(int(gts.sum()), 1), dtype=torch.int64, device=dev)
    error = torch.zeros(1, dtype=torch.int32, device=dev)
    with N.on_device(dev):
        overlaps(scratch, table, dets, gts, pixels, None, order, None, None, inter, int(pairs.sum()), pa,
                 int(dets.sum()), ga, int(gts.sum()), error, N.stream_handle(dev), method="tensor", plan=plan)
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
    sizes = [10 * 101 * C * 12, 10 * C * 12, 12]  # precision, recall, summaries: views of one allocation
    precision, recall, summary = torch.empty(sum(sizes), dtype=torch.float64, device=dev).split(sizes)
    precision = precision.view(10, 101, C, 4, 3)
    recall = recall.view(10, C, 4, 3)
    ws = scratch.get("acc_ws", N.size("pe_instance_accumulate_workspace", n, C), torch.uint8)
    stream = N.stream_handle(dev)
    with N.on_device(dev):
        N.call("pe_instance_accumulate", N.ptr(store.classes), N.ptr(store.ranks), N.ptr(store.flags), 1, CHAINS,
               N.ptr(store.scores), n, N.ptr(counts), C, N.ptr(ws), ws.numel(), N.ptr(precision), N.ptr(recall),
               N.ptr(summary), stream)
    return summarize(precision, recall, summary)
