"""Uneven-size batches: one device arena per batch of images.

``SegmentationImages`` packs many images of different sizes, slot counts and
detection counts into a single byte arena, laid out for the batched kernels:

* target and prediction slot maps: int32, each image starting on a 128-byte
  boundary (16-byte vector loads stay aligned);
* detection masks: one byte per pixel, each mask row padded to a multiple of
  128 bytes (zero padding);
* flat metadata: target classes / crowd [sum G], prediction classes [sum P],
  detection classes / scores [sum D], optional annotation areas [sum G].

The arena exists twice: in pinned host memory (``host``) and on the device
(``device``), with identical offsets, so moving a whole batch to the GPU is a
single ``cudaMemcpyAsync`` (``upload``). The descriptor table that the kernels
read is built once per arena and reused by every update and CUDA-graph replay.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np
import torch

from ._batch import (CHUNK_BEGIN, D, DET_BEGIN, DPAIR_BEGIN, FLAGS, G, MASK_STRIDE, MASKS, P, PAIR_BEGIN, PIXELS,
                     PRED, PSLOT_BEGIN, SEG_CHUNK, SLOT_BEGIN, TARGET, DescTable, Scratch, pass_bounds)
from . import _native as N

ALIGN = 128


def _round(x, a=ALIGN):
    return (x + a - 1) // a * a


@dataclass
class _Field:
    offset: int
    count: int
    dtype: np.dtype


class SegmentationImages:
    """A batch of uneven images for ``SegmentationEvaluator.update_images``."""

    def __init__(self, targets, target_classes, crowd, preds, pred_classes, det_masks, det_classes, scores,
                 instance_areas=None, *, device="cuda", pin=True):
        """Each argument is a list with one numpy array per image (H x W maps, N x H x W bool masks)."""
        B = len(targets)
        self.B = B
        self.hw = np.array([t.shape[0] * t.shape[1] for t in targets], np.int64)
        self.shapes = [tuple(t.shape) for t in targets]
        self.G = np.array([len(c) for c in target_classes], np.int64)
        self.P = np.array([len(c) for c in pred_classes], np.int64)
        self.D = np.array([len(m) for m in det_masks], np.int64)
        self.pitch = np.array([_round(int(n)) for n in self.hw], np.int64)
        layout, cursor = {}, 0

        def reserve(name, count, dtype):
            nonlocal cursor
            cursor = _round(cursor)
            layout[name] = _Field(cursor, int(count), np.dtype(dtype))
            cursor += int(count) * np.dtype(dtype).itemsize

        map_len = int(sum(_round(int(n) * 4) // 4 for n in self.hw))
        reserve("target", map_len, np.int32)
        reserve("pred", map_len, np.int32)
        reserve("masks", int((self.D * self.pitch).sum()), np.uint8)
        reserve("target_classes", self.G.sum(), np.int32)
        reserve("crowd", self.G.sum(), np.uint8)
        reserve("pred_classes", self.P.sum(), np.int32)
        reserve("det_classes", self.D.sum(), np.int32)
        reserve("scores", self.D.sum(), np.float64)
        self.has_areas = instance_areas is not None
        if self.has_areas:
            reserve("areas", self.G.sum(), np.float64)
        self.nbytes = _round(cursor)
        self.layout = layout
        self.host = torch.empty(self.nbytes, dtype=torch.uint8, pin_memory=pin)
        buf = self.host.numpy()
        self.map_offset = np.zeros(B, np.int64)  # element offsets into the map arrays
        self.mask_offset = np.zeros(B, np.int64)  # byte offsets into the mask array
        m_off, k_off = 0, 0
        views = {name: self._host_view(buf, f) for name, f in layout.items()}
        for b in range(B):
            n = int(self.hw[b])
            self.map_offset[b] = m_off
            views["target"][m_off:m_off + n] = targets[b].reshape(-1)
            views["pred"][m_off:m_off + n] = preds[b].reshape(-1)
            m_off += _round(n * 4) // 4
            self.mask_offset[b] = k_off
            rows = views["masks"][k_off:k_off + int(self.D[b] * self.pitch[b])].reshape(int(self.D[b]),
                                                                                     int(self.pitch[b]))
            if self.D[b]:
                rows[:, :n] = det_masks[b].reshape(int(self.D[b]), n)
                rows[:, n:] = 0
            k_off += int(self.D[b] * self.pitch[b])
        for name, parts in (("target_classes", target_classes), ("crowd", crowd), ("pred_classes", pred_classes),
                            ("det_classes", det_classes), ("scores", scores)):
            views[name][:] = np.concatenate([np.asarray(p).reshape(-1) for p in parts]) if B else 0
        if self.has_areas:
            views["areas"][:] = np.concatenate([np.asarray(a, np.float64).reshape(-1) for a in instance_areas])
        self.device = torch.empty(self.nbytes, dtype=torch.uint8, device=device)
        self.upload()
        self._table = None

    @staticmethod
    def _host_view(buf, field):
        return buf[field.offset: field.offset + field.count * field.dtype.itemsize].view(field.dtype)

    def tensor(self, name):
        """Device view of one field."""
        f = self.layout[name]
        torch_dtype = {np.dtype(np.int32): torch.int32, np.dtype(np.uint8): torch.uint8,
                       np.dtype(np.float64): torch.float64}[f.dtype]
        return self.device[f.offset: f.offset + f.count * f.dtype.itemsize].view(torch_dtype)

    def upload(self):
        """Copy the whole host arena to the device on the current stream (asynchronous)."""
        self.device.copy_(self.host, non_blocking=True)
        return self

    @property
    def bytes_per_batch(self):
        return self.nbytes

    def algorithmic_bytes(self):
        """Bytes the fused pass must read: 8 per pixel (two int32 maps) + 1 per detection pixel."""
        return int((self.hw * (8 + self.D)).sum())

    def table(self, scratch: Scratch):
        if self._table is None:
            B = self.B
            t = DescTable(B)
            d = t.desc
            base = self.device.data_ptr()
            d[:, TARGET] = base + self.layout["target"].offset + 4 * self.map_offset
            d[:, PRED] = base + self.layout["pred"].offset + 4 * self.map_offset
            d[:, MASKS] = base + self.layout["masks"].offset + self.mask_offset
            d[:, PIXELS] = self.hw
            d[:, MASK_STRIDE] = self.pitch
            chunks = -(-self.hw // SEG_CHUNK)
            d[:, CHUNK_BEGIN] = np.cumsum(chunks) - chunks
            d[:, DET_BEGIN] = np.cumsum(self.D) - self.D
            d[:, SLOT_BEGIN] = np.cumsum(self.G) - self.G
            d[:, PSLOT_BEGIN] = np.cumsum(self.P) - self.P
            pan = self.G * self.P
            d[:, PAIR_BEGIN] = np.cumsum(pan) - pan
            det = self.D * self.G
            d[:, DPAIR_BEGIN] = np.cumsum(det) - det
            d[:, D] = self.D
            d[:, G] = self.G
            d[:, P] = self.P
            d[:, FLAGS] = 3  # maps and mask rows are 128-byte aligned by construction
            t.total_chunks = int(chunks.sum())
            # Fused-pass CTA ranges of equal bytes (2 CTAs per SM): images differ widely in detections.
            t.finish(scratch, f"ragged_descs_{id(self)}",
                     bounds=pass_bounds(self.hw, self.D, 2 * N.sm_count(self.device.device)))
            self._table = t
        return self._table
