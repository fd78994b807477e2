"""Joint PQ/mIoU and mask AP/AR with one shared panoptic target (API of the reference's combined.py).

One ``update`` over a batch is five launches, independent of the number of
images: per-image score sort, one fused pass over the pixels (panoptic pair
histogram + detection x target-slot histogram), per-image scoring (areas and
validation, then PQ/confusion accumulation), and batched COCO matching. With
``validate=False`` nothing synchronises with the host, so an update can be
captured in a CUDA graph.
"""

from __future__ import annotations

from dataclasses import replace
from typing import Sequence

import numpy as np
import torch

from . import _native as N
from ._batch import (CHAINS, CHUNK_BEGIN, D, DET_BEGIN, DPAIR_BEGIN, FLAGS, G, MASK_STRIDE, MASKS, P, PAIR_BEGIN,
                     PIXELS, PRED, PSLOT_BEGIN, SEG_CHUNK, SLOT_BEGIN, TARGET, DescTable, aligned, pass_bounds)
from .evaluator import PanopticBatch, PanopticEvaluator, _prepare, raise_validation
from .instance import InstanceBatch, InstanceEvaluator, check_instance_batch

# The fused pass streams mask rows through a bulk-copy ring (rows at any
# alignment; set False to force the register-prefetch pass) ...
BULK_PASS = True
# ... and hands out its chunks from a device counter, so faster CTAs take more of
# them (set False for the host-computed contiguous range of equal bytes per CTA).
DYNAMIC_PASS = True

# Benchmark hook: when a list, each update appends (start, end) CUDA events
# recorded around the fused pixel pass on the launching stream.
PASS_EVENTS = None

_COMBINED_ERRORS = (
    (32, "scores must be finite; areas must be nonnegative"),
    (64, "instance_areas must be finite and nonnegative"),
    (8, "detection categories must be thing classes"),
    (16, "each instance mask must have pixels"),
)


class SegmentationEvaluator:
    """PQ/mIoU and mask AP/AR with separate predictions and one shared target (combined.py:18-167).

    AP ground truth is exactly the thing segments of the panoptic target.
    """

    def __init__(self, num_classes: int, *, isthing: Sequence[bool] | None = None,
                 device: str | torch.device = "cuda", validate: bool = True):
        self.panoptic = PanopticEvaluator(num_classes, isthing=isthing, device=device, validate=validate)
        self.device = self.panoptic.tp.device
        self.instance = InstanceEvaluator(num_classes, device=self.device, validate=validate)
        self.num_classes = num_classes
        self.validate = validate
        self._isthing_u8 = self.panoptic.isthing.to(torch.uint8)
        # Stream of the panoptic half of compute(), made here rather than during a graph capture.
        self._side = torch.cuda.Stream(self.device) if self.device.type == "cuda" else None

    def reset(self):
        self.panoptic.reset()
        self.instance.reset()

    def state_dict(self) -> dict:
        """Panoptic counters under ``panoptic/`` and instance records / positives under ``instance/``."""
        state = {f"panoptic/{k}": v for k, v in self.panoptic.state_dict().items()}
        state.update({f"instance/{k}": v for k, v in self.instance.state_dict().items()})
        return state

    def load_state_dict(self, state: dict):
        self.panoptic.load_state_dict({k.split("/", 1)[1]: v for k, v in state.items() if k.startswith("panoptic/")})
        self.instance.load_state_dict({k.split("/", 1)[1]: v for k, v in state.items() if k.startswith("instance/")})
        return self

    def _check_areas(self, areas, classes):
        if areas is None:
            return None
        if areas.shape != classes.shape or areas.device != self.device or not areas.is_floating_point():
            raise ValueError("instance_areas must be floating point B x S on evaluator device")
        return areas.to(torch.float64).contiguous()

    @torch.no_grad()
    def update(self, prediction: PanopticBatch, detections: InstanceBatch, target: PanopticBatch, *,
               instance_areas: torch.Tensor | None = None):
        """Accumulate all metrics; optional annotation areas have shape B x S (combined.py:63-161)."""
        target = target.compact()
        prediction = prediction.compact()
        if target.crowd is None:
            target = replace(target, crowd=torch.zeros_like(target.classes, dtype=torch.bool))
        maps, classes, crowd = _prepare(target, self.num_classes)
        pred, pc, _ = _prepare(prediction, self.num_classes, ignore_crowd=True)
        if maps.device != self.device:
            raise ValueError("target must share evaluator device")
        if pred.shape != maps.shape or pred.device != maps.device:
            raise ValueError("prediction and target must share shape and evaluator device")
        check_instance_batch(detections, self.device, prediction=True)
        if len(detections.masks) != maps.shape[0] or any(m.shape[1:] != maps.shape[1:] for m in detections.masks):
            raise ValueError("detections and target must have matching image counts and dimensions")
        ann = self._check_areas(instance_areas, classes)
        B, H, W = maps.shape
        if B == 0:
            return self
        masks = [m.contiguous() for m in detections.masks]
        run_batch(self, maps, pred, classes, pc, crowd, masks, detections.classes, detections.scores, ann,
                  [H * W] * B)
        return self

    @torch.no_grad()
    def update_images(self, images):
        """Accumulate a batch of uneven images packed in a ``ragged.SegmentationImages`` arena.

        The arena's descriptor table is reused, so with ``validate=False`` this
        call launches the same five kernels with the same pointers every time
        and can be captured in a CUDA graph.
        """
        if images.device.device != self.device:
            raise ValueError("images must live on the evaluator device")
        if images.B == 0:
            return self
        table = images.table(self.instance._scratch)
        launch(self, table, images.tensor("target_classes"), images.tensor("pred_classes"), images.tensor("crowd"),
               images.tensor("det_classes"), images.tensor("scores"),
               images.tensor("areas") if images.has_areas else None)
        return self

    def compute(self):
        """Panoptic/semantic results plus an 'instance' AP/AR dictionary (combined.py:163-167).

        The panoptic summary (one CTA) runs on a side stream beside the AP
        accumulation chain on the current stream; the current stream waits for
        both before this returns, so callers see one ordered stream (and a CUDA
        graph capture sees a fork and a join).
        """
        side = self._side
        if side is None:
            result = self.panoptic.compute()
            result["instance"] = self.instance.compute()
            return result
        main = torch.cuda.current_stream(self.device)
        side.wait_stream(main)
        with torch.cuda.stream(side):
            result = self.panoptic.compute()
        result["instance"] = self.instance.compute()
        main.wait_stream(side)
        # The panoptic outputs are views of two allocations made on the side stream (FP64 values, int64
        # counts): the caching allocator must not hand them out again before the current stream's later
        # uses are done.
        result["miou"].record_stream(main)
        result["tp"].record_stream(main)
        return result


def run_batch(ev: SegmentationEvaluator, maps, pred, classes, pc, crowd, masks, det_classes, det_scores, ann,
              pixels):
    """Launch the batched pipeline for B images of a (B x H x W)-shaped batch."""
    B = len(masks)
    HW = pixels[0]
    S, Pn = classes.shape[1], pc.shape[1]
    dets = np.array([m.shape[0] for m in masks], np.int64)
    table = DescTable(B)
    d = table.desc
    img = np.arange(B, dtype=np.int64)
    d[:, TARGET] = maps.data_ptr() + img * HW * 4
    d[:, PRED] = pred.data_ptr() + img * HW * 4
    d[:, MASKS] = [m.data_ptr() for m in masks]
    d[:, PIXELS] = HW
    d[:, MASK_STRIDE] = HW
    chunks = -(-HW // SEG_CHUNK)
    d[:, CHUNK_BEGIN] = img * chunks
    d[:, DET_BEGIN] = np.cumsum(dets) - dets
    d[:, SLOT_BEGIN] = img * S
    d[:, PSLOT_BEGIN] = img * Pn
    d[:, PAIR_BEGIN] = img * S * Pn
    dp = dets * S
    d[:, DPAIR_BEGIN] = np.cumsum(dp) - dp
    d[:, D] = dets
    d[:, G] = S
    d[:, P] = Pn
    maps_vec = aligned(maps.data_ptr()) and aligned(pred.data_ptr()) and HW % 4 == 0
    d[:, FLAGS] = [int(maps_vec) | 2 * int(aligned(m.data_ptr(), HW)) for m in masks]
    table.total_chunks = int(chunks * B)
    table.finish(ev.instance._scratch, "seg_descs", bounds=pass_bounds(np.full(B, HW), dets, 2 * N.sm_count(ev.device)))
    total_d = int(dets.sum())
    dev = ev.device
    dc = torch.cat([c.reshape(-1).to(torch.int32) for c in det_classes]) if total_d else \
        torch.empty(0, dtype=torch.int32, device=dev)
    ds = torch.cat([s.reshape(-1).to(torch.float64) for s in det_scores]) if total_d else \
        torch.empty(0, dtype=torch.float64, device=dev)
    launch(ev, table, classes.reshape(-1), pc.reshape(-1), crowd.reshape(-1).view(torch.uint8), dc, ds,
           ann.reshape(-1) if ann is not None else None)


def launch(ev, table, gc, pc, crowd_u8, det_classes, det_scores, ann):
    """Shared launch sequence over a finished descriptor table and flat metadata tensors."""
    dev = ev.device
    inst, pan = ev.instance, ev.panoptic
    Sc = inst._scratch
    C = ev.num_classes
    desc = table.desc
    B = table.B
    total_d = int(desc[:, D].sum())
    slots_total, pslots_total = int(desc[:, G].sum()), int(desc[:, P].sum())
    max_g, max_p = int(max(desc[:, G].max(), 1)), int(max(desc[:, P].max(), 1))
    store = inst._store
    store.reserve(total_d)
    out_scores, out_classes, out_ranks, out_flags = store.tail()
    error = Sc.get("error", 1, torch.int32, zero=True)
    order = Sc.get("order", total_d, torch.int64)
    ws = Sc.get("sort_ws", N.size("pe_seg_sort_workspace", total_d), torch.uint8)
    pairs_len = int(desc[:, G] @ desc[:, P])
    dpairs_len = int(desc[:, D] @ desc[:, G])
    pairs = Sc.get("pairs", pairs_len, torch.int32)
    dpairs = Sc.get("dpairs", dpairs_len, torch.int32)
    areas = Sc.get("areas", slots_total + pslots_total, torch.int64)
    matched = Sc.get("matched", slots_total, torch.int32)
    det_pa = Sc.get("det_pa", total_d, torch.float64)
    slot_ga = Sc.get("slot_ga", slots_total, torch.float64)
    slot_class = Sc.get("slot_class", slots_total, torch.int32)
    ann_out = Sc.get("ann", slots_total, torch.float64)
    class_bits = Sc.get("class_bits", B * ((C + 31) // 32), torch.int32)
    stream = N.stream_handle(dev)
    pan_cap = int((desc[:, G] * desc[:, P]).max())
    det_cap = int((desc[:, D] * desc[:, G]).max())
    with N.on_device(dev):
        N.call("pe_seg_sort", N.ptr(table.descs), B, N.ptr(det_scores), N.ptr(det_classes), total_d, N.ptr(order),
               N.ptr(out_scores), N.ptr(out_classes), N.ptr(ws), ws.numel(), stream)
        if PASS_EVENTS is not None:
            events = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
            events[0].record()
        # 1: every mask row starts on a 16-byte boundary; 2: rows at any offset (re-aligned in the pass).
        bulk = (1 if bool((desc[:, FLAGS] & 2).all()) else 2) if BULK_PASS else 0
        bounds = getattr(table, "bounds", None) if bulk else None
        schedule = Sc.get("pass_schedule", 1, torch.int64) if bulk and DYNAMIC_PASS else None
        N.call("pe_seg_pass", N.ptr(table.descs), B, table.total_chunks, N.ptr(order), N.ptr(pairs), pairs_len,
               N.ptr(dpairs), dpairs_len, pan_cap, det_cap, bulk, N.ptr(bounds), table.ctas if bounds is not None else 0,
               N.ptr(schedule), N.ptr(error), stream)
        if PASS_EVENTS is not None:
            events[1].record()
            PASS_EVENTS.append(events)
        N.call("pe_seg_score", N.ptr(table.descs), B, max_p, pan_cap, N.ptr(pairs), N.ptr(dpairs), N.ptr(gc),
               N.ptr(pc), N.ptr(crowd_u8), N.ptr(areas), N.ptr(matched), N.ptr(pan.tp), N.ptr(pan.fp), N.ptr(pan.fn),
               N.ptr(pan.iou_sum), N.ptr(pan.confusion), C, N.ptr(ev._isthing_u8), N.ptr(out_classes),
               N.ptr(out_scores), N.ptr(det_pa), N.ptr(slot_ga), N.ptr(slot_class), N.ptr(ann), N.ptr(ann_out),
               int(ev.validate), 0, N.ptr(class_bits), N.ptr(error), stream)
        N.call("pe_seg_match", N.ptr(dpairs), N.ptr(table.pair_off), N.ptr(table.d_off), N.ptr(table.g_off), B,
               N.ptr(out_classes), N.ptr(det_pa), N.ptr(slot_class), N.ptr(slot_ga), N.ptr(crowd_u8), N.ptr(ann_out),
               C, max_g, N.ptr(out_flags), 1, CHAINS, N.ptr(out_ranks), N.ptr(inst._counts), N.ptr(error),
               N.ptr(class_bits), stream)
    if ev.validate:
        code = int(error.item())
        if code & (8 | 16 | 32 | 64):
            for bit, message in _COMBINED_ERRORS:
                if code & bit:
                    raise ValueError(message)
        raise_validation(code)
    store.n += total_d
