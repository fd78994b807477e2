"""Panoptic quality, semantic mIoU and per-image reward PQ on CUDA.

Same public API and semantics as the reference's ``panoptic_evaluator/evaluator.py``
(``PanopticBatch``, ``PanopticEvaluator``, ``panoptic_quality``); every pixel
and segment computation runs in the sm_103a kernels of ``libpe_gb300.so``.
Tensors must live on a CUDA device: this package has no CPU path.
"""

from __future__ import annotations

from dataclasses import dataclass, replace
from numbers import Integral
from typing import Sequence

import numpy as np
import torch

from . import _cuda_evaluator as native
from . import _native as N

_INT64_MAX = torch.iinfo(torch.int64).max
_MESSAGES = {
    1: "map contains an unknown segment ID or a slot outside metadata capacity",
    2: "classes must be -1 or valid category indices; slot 0 must be void",
    4: "nonvoid map slots and active metadata must correspond exactly",
}


def _require_cuda(tensor, what="inputs"):
    if not tensor.is_cuda:
        raise ValueError(f"{what} must be CUDA tensors: pe_gb300 evaluates on the GPU only")


def raise_validation(code: int):
    """Turn a validation bitmask into the reference's ValueError (evaluator.py:365-376)."""
    if code:
        for bit in (1, 2, 4):
            if code & bit:
                raise ValueError(_MESSAGES[bit])
        raise ValueError(f"invalid input (code {code})")


@dataclass(frozen=True)
class PanopticBatch:
    """Segment maps and metadata; optional lookup tables allow original IDs (evaluator.py:23-31)."""

    segment_map: torch.Tensor  # B x H x W; compact int32 or original int32/int64 IDs
    classes: torch.Tensor  # B x S int32; slot 0 is void, class -1 is padding
    crowd: torch.Tensor | None = None  # B x S bool; ground truth only
    lookup_ids: torch.Tensor | None = None  # B x S sorted int64 original IDs
    lookup_slots: torch.Tensor | None = None  # B x S int32 original metadata slots

    @classmethod
    def from_coco(cls, maps: torch.Tensor, segments_info: Sequence[Sequence[dict]], category_ids: Sequence[int],
                  *, compact: bool = True) -> "PanopticBatch":
        """Build slot tables from COCO ``segments_info`` (evaluator.py:33-106).

        Metadata keeps input order (official crowd semantics). All tables are
        uploaded with a single host-to-device copy. ``compact=False`` keeps the
        original IDs and resolves them inside the histogram pass. ``maps`` may
        also be the decoded COCO panoptic PNGs, B x H x W x 3 uint8 RGB: IDs are
        R + 256 G + 65536 B, decoded on the GPU (fused with the slot lookup
        when compacting).
        """
        if _is_rgb(maps):
            if not compact:
                maps = decode_rgb(maps)
        elif maps.ndim != 3 or maps.dtype not in (torch.int32, torch.int64):
            raise ValueError("maps must be integer B x H x W tensors (or uint8 B x H x W x 3 RGB)")
        if len(segments_info) != maps.shape[0] or len(set(category_ids)) != len(category_ids):
            raise ValueError("batch length or category IDs are invalid")
        index = {category: i for i, category in enumerate(category_ids)}
        B = maps.shape[0]
        S = max((len(info) for info in segments_info), default=0) + 1
        ids = np.full((B, S), _INT64_MAX, np.int64)
        slots = np.zeros((B, S), np.int32)
        classes = np.full((B, S), -1, np.int32)
        crowd = np.zeros((B, S), np.bool_)
        for b, info in enumerate(segments_info):
            segment_ids = [entry["id"] for entry in info]
            if (any(not isinstance(i, Integral) or isinstance(i, bool) or i <= 0 or i >= _INT64_MAX
                    for i in segment_ids) or len(set(segment_ids)) != len(segment_ids)):
                raise ValueError("segment IDs must be unique positive int64 values below INT64_MAX; 0 is void")
            try:
                labels = [index[entry["category_id"]] for entry in info]
            except KeyError as error:
                raise ValueError("unknown category_id") from error
            n = len(info)
            classes[b, 1:n + 1] = labels
            crowd[b, 1:n + 1] = [bool(entry.get("iscrowd", 0)) for entry in info]
            ordered = sorted(zip(segment_ids, range(1, n + 1)))
            ids[b, 0] = 0
            ids[b, 1:n + 1] = [int(i) for i, _ in ordered]
            slots[b, 1:n + 1] = [s for _, s in ordered]
        # One upload: int64 then int32 fields, bool last, viewed out of one buffer.
        fields = (ids, slots, classes, crowd)
        host = np.concatenate([f.reshape(-1).view(np.uint8) for f in fields])
        storage = torch.from_numpy(host).to(maps.device)
        views, offset = [], 0
        for field, dtype in zip(fields, (torch.int64, torch.int32, torch.int32, torch.bool)):
            size = field.nbytes
            views.append(storage[offset:offset + size].view(dtype).reshape(B, S))
            offset += size
        lookup_ids, lookup_slots, table_classes, table_crowd = views
        batch = cls(maps, table_classes, table_crowd, lookup_ids, lookup_slots)
        return batch.compact() if compact else batch

    def with_maps(self, maps: torch.Tensor) -> "PanopticBatch":
        """Reuse prepared metadata for another map batch (evaluator.py:108-118); RGB maps are decoded to IDs."""
        if _is_rgb(maps):
            if self.lookup_ids is None:
                raise ValueError("RGB maps carry original IDs: build the batch with from_coco first")
            maps = decode_rgb(maps)
        if maps.ndim != 3 or maps.shape[0] != self.classes.shape[0] or maps.device != self.classes.device:
            raise ValueError("new maps must have the same batch size and metadata device")
        return replace(self, segment_map=maps)

    def compact(self) -> "PanopticBatch":
        """Materialise compact slots with one pixel kernel (evaluator.py:120-158)."""
        if self.lookup_ids is None:
            return self
        maps = self.segment_map
        rgb = _is_rgb(maps)
        if not rgb and (maps.ndim != 3 or maps.dtype not in (torch.int32, torch.int64)):
            raise ValueError("maps must be integer B x H x W tensors")
        if (self.lookup_slots is None or self.lookup_ids.shape != self.classes.shape
                or self.lookup_slots.shape != self.classes.shape):
            raise ValueError("lookup IDs and slots must match classes shape")
        if (self.lookup_ids.device != maps.device or self.lookup_slots.device != maps.device
                or maps.shape[0] != self.classes.shape[0]):
            raise ValueError("lookup tables and maps must share device and batch size")
        _require_cuda(maps, "segment maps")
        if rgb:
            packed, error = _pack_rgb(maps.contiguous(), self.lookup_ids.contiguous(), self.lookup_slots.contiguous())
        else:
            packed, error = native.pack(maps.contiguous(), self.lookup_ids.contiguous(),
                                        self.lookup_slots.contiguous())
        if error.item():
            raise ValueError("map contains a segment absent from segments_info")
        return PanopticBatch(packed, self.classes, self.crowd)


def _is_rgb(maps: torch.Tensor) -> bool:
    return maps.ndim == 4 and maps.shape[-1] == 3 and maps.dtype == torch.uint8


def _pack_rgb(rgb: torch.Tensor, ids, slots):
    B, H, W, _ = rgb.shape
    out = torch.empty((B, H, W), dtype=torch.int32, device=rgb.device)
    error = torch.zeros(1, dtype=torch.int32, device=rgb.device)
    with torch.cuda.device(rgb.device):
        N.call("pe_pack_rgb", N.ptr(rgb), B, H * W, N.ptr(ids), N.ptr(slots), 0 if ids is None else ids.shape[1],
               N.ptr(out), N.ptr(error), N.stream_handle(rgb.device))
    return out, error


def decode_rgb(rgb: torch.Tensor) -> torch.Tensor:
    """Decoded COCO panoptic PNGs (B x H x W x 3 uint8 RGB, CUDA) -> int32 IDs R + 256 G + 65536 B."""
    if not _is_rgb(rgb):
        raise ValueError("RGB maps must be uint8 B x H x W x 3 tensors")
    _require_cuda(rgb, "RGB maps")
    if rgb.shape[0] > 65535:
        return torch.cat([decode_rgb(part) for part in rgb.split(65535)])
    return _pack_rgb(rgb.contiguous(), None, None)[0]


def _prepare(batch: PanopticBatch, num_classes: int, *, ignore_crowd: bool = False):
    """Shape/dtype/device checks (evaluator.py:161-207). Value checks run on the GPU."""
    maps, classes = batch.segment_map, batch.classes
    if maps.ndim != 3 or classes.ndim != 2 or classes.shape[0] != maps.shape[0] or classes.shape[1] < 1:
        raise ValueError("expected maps B x H x W and classes B x S with S >= 1")
    original_ids = batch.lookup_ids is not None
    if (batch.lookup_slots is not None) != original_ids:
        raise ValueError("lookup IDs and slots must be supplied together")
    map_dtypes = (torch.int32, torch.int64) if original_ids else (torch.int32,)
    if maps.dtype not in map_dtypes or classes.dtype != torch.int32:
        raise ValueError("classes and compact maps must be int32; original ID maps may also be int64")
    if original_ids:
        for lookup, dtype in ((batch.lookup_ids, torch.int64), (batch.lookup_slots, torch.int32)):
            if lookup.shape != classes.shape or lookup.dtype != dtype or lookup.device != maps.device:
                raise ValueError("lookup tables must match metadata shape, device and expected dtypes")
    crowd = None
    if not ignore_crowd:
        crowd = batch.crowd if batch.crowd is not None else torch.zeros_like(classes, dtype=torch.bool)
        if crowd.shape != classes.shape or crowd.dtype != torch.bool:
            raise ValueError("crowd must be bool with the same shape as classes")
    if classes.device != maps.device or (crowd is not None and crowd.device != maps.device):
        raise ValueError("batch tensors must share a device")
    _require_cuda(maps, "segment maps")
    return maps.contiguous(), classes.contiguous(), crowd.contiguous() if crowd is not None else None


def _tables(batch):
    if batch.lookup_ids is None:
        return None, None
    return batch.lookup_ids.contiguous(), batch.lookup_slots.contiguous()


class PanopticEvaluator:
    """Dataset PQ/SQ/RQ and semantic IoU accumulated on the GPU (evaluator.py:246-468)."""

    def __init__(self, num_classes: int, *, isthing: Sequence[bool] | None = None,
                 device: str | torch.device = "cuda", validate: bool = True):
        if not isinstance(num_classes, int) or isinstance(num_classes, bool) or num_classes <= 0:
            raise ValueError("num_classes must be a positive integer")
        if isthing is not None and len(isthing) != num_classes:
            raise ValueError("isthing must contain one flag per category")
        self.num_classes = num_classes
        self.device = torch.device(device)
        if self.device.type != "cuda":
            raise ValueError("pe_gb300 evaluates on CUDA devices only")
        self.validate = validate
        self.isthing = torch.tensor(isthing if isthing is not None else [True] * num_classes, dtype=torch.bool,
                                    device=self.device)
        self._scratch = None
        self._default_crowd = None
        self._validation_error = torch.zeros(1, dtype=torch.int32, device=self.device)
        self.reset()

    def reset(self):
        if hasattr(self, "_state"):
            self._state.zero_()  # one fill clears every accumulator (0.0 is the all-zero bit pattern)
            return
        C = self.num_classes
        # tp, fp, fn [C], iou_sum [C] (float64) and confusion [C, C + 1] are views of one allocation. The last
        # confusion column counts predicted void on valid ground-truth pixels.
        self._state = torch.zeros(4 * C + C * (C + 1), dtype=torch.int64, device=self.device)
        tp, fp, fn, sums, confusion = self._state.split([C, C, C, C, C * (C + 1)])
        self.tp, self.fp, self.fn = tp, fp, fn
        self.iou_sum = sums.view(torch.float64)
        self.confusion = confusion.view(C, C + 1)

    STATE = ("tp", "fp", "fn", "iou_sum", "confusion")

    def state_dict(self) -> dict:
        """Accumulated state (copies): tp, fp, fn, iou_sum, confusion."""
        return {key: getattr(self, key).clone() for key in self.STATE}

    def load_state_dict(self, state: dict):
        """Replace the accumulated state (for example with replicas merged by ``distributed``)."""
        for key in self.STATE:
            value = state[key]
            target = getattr(self, key)
            if value.shape != target.shape:
                raise ValueError(f"{key}: expected shape {tuple(target.shape)}, got {tuple(value.shape)}")
            target.copy_(value.to(device=target.device, dtype=target.dtype))
        return self

    @torch.no_grad()
    def update(self, prediction: PanopticBatch, target: PanopticBatch):
        return self._update(prediction, target)

    def _scratch_for(self, B, G, P, device):
        shape = (B, G, P)
        if self._scratch is None or tuple(self._scratch[0].shape) != shape:
            self._scratch = (torch.empty(shape, dtype=torch.int64, device=device),
                             torch.empty((B, G + P), dtype=torch.int64, device=device),
                             torch.empty((B, G), dtype=torch.int32, device=device))
        return self._scratch

    @torch.no_grad()
    def _update(self, prediction: PanopticBatch, target: PanopticBatch, *, return_areas=False):
        if target.crowd is None and target.segment_map.is_cuda:
            if (self._default_crowd is None or self._default_crowd.shape != target.classes.shape
                    or self._default_crowd.device != target.classes.device):
                self._default_crowd = torch.zeros_like(target.classes, dtype=torch.bool)
            target = replace(target, crowd=self._default_crowd)
        gt, gc, crowd = _prepare(target, self.num_classes)
        pred, pc, _ = _prepare(prediction, self.num_classes, ignore_crowd=True)
        if gt.shape != pred.shape or gt.device != pred.device or gt.device != self.tp.device:
            raise ValueError("prediction and target must share shape and evaluator device")
        B, G, P = gt.shape[0], gc.shape[1], pc.shape[1]
        scratch = self._scratch_for(B, G, P, gt.device)
        gi, gs = _tables(target)
        pi, ps = _tables(prediction)
        if gi is None and pi is None:
            # Compact maps: the inputs were checked by _prepare and the state and scratch are this evaluator's
            # own, so the C ABI is called directly (it checks the sizes) without the extension shim's checks.
            with N.on_device(gt.device):
                code = N.call("pe_update", gt.data_ptr(), 0, pred.data_ptr(), 0, B, gt.shape[1] * gt.shape[2],
                              gc.data_ptr(), pc.data_ptr(), crowd.data_ptr(), G, P, self.num_classes,
                              scratch[0].data_ptr(), scratch[1].data_ptr(), scratch[2].data_ptr(),
                              self.tp.data_ptr(), self.fp.data_ptr(), self.fn.data_ptr(), self.iou_sum.data_ptr(),
                              self.confusion.data_ptr(), None, None, None, None, self._validation_error.data_ptr(),
                              int(bool(self.validate)), 0, N.stream_handle(gt.device))
        else:
            code = native.update(gt, pred, gc, pc, crowd, *scratch, self.tp, self.fp, self.fn, self.iou_sum,
                                 self.confusion, gi, gs, pi, ps, self._validation_error, self.validate)
        raise_validation(code)
        return scratch[1][:, :G] if return_areas else self

    @torch.no_grad()
    def compute(self) -> dict:
        """Device tensors in [0, 1]; absent classes have zero PQ and NaN IoU (evaluator.py:419-447)."""
        rows, s, n, miou, copies = native.compute_one(self.tp, self.fp, self.fn, self.iou_sum, self.confusion,
                                                      self.isthing, self.num_classes)
        tp, fp, fn, sums, confusion = copies
        result = {name: {"pq": s[3 * i], "sq": s[3 * i + 1], "rq": s[3 * i + 2], "n": n[i]}
                  for i, name in enumerate(("All", "Things", "Stuff"))}
        result.update(per_class=dict(zip(("pq", "sq", "rq", "iou"), rows)), miou=miou, tp=tp, fp=fp, fn=fn,
                      iou_sum=sums, confusion=confusion)
        return result


@torch.no_grad()
def panoptic_quality(prediction: PanopticBatch, target: PanopticBatch, num_classes: int, reduction: str = "none",
                     *, validate: bool = True, return_stats: bool = False) -> torch.Tensor:
    """Stateless mean-class PQ per image, float64 on the input device (evaluator.py:471-544).

    Prediction slots without pixels are ignored. ``return_stats=True`` returns
    [image, class, (IoU sum, TP, FP, FN)] statistics instead of scores.
    """
    if not isinstance(num_classes, int) or isinstance(num_classes, bool) or num_classes <= 0:
        raise ValueError("num_classes must be a positive integer")
    if reduction != "none":
        raise ValueError('reduction must be "none"')
    gt, gc, crowd = _prepare(target, num_classes)
    pred, pc, _ = _prepare(prediction, num_classes, ignore_crowd=True)
    if gt.shape != pred.shape or gt.device != pred.device:
        raise ValueError("prediction and target must share shape and device")
    stats = reward_statistics(gt, pred, gc, pc, crowd, num_classes, _tables(target), _tables(prediction), validate)
    if return_stats:
        return stats
    return reward_scores(stats)


def reward_statistics(gt, pred, gc, pc, crowd, num_classes, gt_tables=(None, None), pred_tables=(None, None),
                      validate=True):
    """[B, C, 4] (iou_sum, tp, fp, fn) per image, computed by one pe_update in reward mode."""
    B, G, P = gt.shape[0], gc.shape[1], pc.shape[1]
    device = gt.device
    longs = torch.zeros((3, B, num_classes), dtype=torch.int64, device=device)
    sums = torch.zeros((B, num_classes), dtype=torch.float64, device=device)
    code = native.update(gt, pred, gc, pc, crowd,
                         torch.empty((B, G, P), dtype=torch.int64, device=device),
                         torch.empty((B, G + P), dtype=torch.int64, device=device),
                         torch.empty((B, G), dtype=torch.int32, device=device),
                         longs[0], longs[1], longs[2], sums, torch.empty(0, dtype=torch.int64, device=device),
                         *gt_tables, *pred_tables, torch.zeros(1, dtype=torch.int32, device=device), validate,
                         True)
    raise_validation(code)
    return torch.stack((sums, longs[0].double(), longs[1].double(), longs[2].double()), -1)


def reward_scores(stats):
    """Mean over active classes of PQ per image (evaluator.py:539-544)."""
    sums, tp, fp, fn = stats.unbind(-1)
    denominator = tp + 0.5 * (fp + fn)
    active = denominator > 0
    return (sums / denominator.clamp_min(1)).sum(1) / active.sum(1).clamp_min(1)
