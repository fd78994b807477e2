"""Host-side plumbing shared by the batched evaluators.

* ``DescTable`` builds the per-image descriptor table that the batched
  kernels read (layout documented in ``csrc/pe_segmentation.cu``) plus the
  matching offsets, and uploads everything with one pinned async copy.
* ``Scratch`` caches device buffers by name so repeated updates of the same
  shape reuse the same memory (and CUDA-graph captures see stable pointers).
* ``RecordStore`` keeps instance records (score, class, rank, 40 match flags)
  on the device between updates, record-major, growing geometrically.
"""

from __future__ import annotations

import numpy as np
import torch

from . import _native as N

FIELDS = 16
(TARGET, PRED, MASKS, PIXELS, MASK_STRIDE, CHUNK_BEGIN, DET_BEGIN, SLOT_BEGIN, PSLOT_BEGIN, PAIR_BEGIN,
 DPAIR_BEGIN, D, G, P, FLAGS, RESERVED) = range(FIELDS)
SEG_CHUNK = 8192  # pixels per work chunk of the fused pass
INST_CHUNK = 4096  # pixels per chunk of the mask-overlap kernel
CHAINS = 40


CONTRACT_CHUNK = 4096  # pixels per chunk of the tensor-core mask contraction
CONTRACT_ROWS = (127, 63)  # detections x targets per contraction block
# Cost of a TMA-loaded stage relative to a staged one (0.259 vs 0.353 ms for the same 32 COCO-like images).
CONTRACT_TMA_COST = 0.73


def contract_blocks(dets, gts, pixels, ctas=None, tma=None, tma_cost=None):
    """Block table of pe_inst_contract: rows (image, first detection, first target, first chunk).

    Each image with pixels and at least one mask is covered by 127 x 63 tiles
    of ceil(pixels / 4096) chunks. Images loaded by TMA (``tma``, bool per
    image) come after all staged images in chunk order: a CTA's range may go
    from staged to TMA blocks but never back (the kernel's staged stages pace
    every worker warp, TMA stages only the one issuing the loads). With
    `ctas`, also returns ctas + 1 chunk bounds (fewer when there are fewer
    chunks) that give every CTA a contiguous range of about equal cost (mask
    rows x pixels, TMA blocks weighted by `tma_cost`, CONTRACT_TMA_COST by
    default). Planned by pe_contract_blocks on the host. Returns (int64
    [n, 4] array, total chunks[, bounds]).
    """
    dets, gts, pixels = (np.ascontiguousarray(x, np.int64).reshape(-1) for x in (dets, gts, pixels))
    B = dets.size
    flags = None if tma is None else np.ascontiguousarray(tma, np.uint8).reshape(-1)
    rows_a, rows_b = CONTRACT_ROWS
    # At least the blocks of every image (an image without masks of one kind still takes one tile).
    cap = int(((dets + rows_a - 1) // rows_a + 1) @ ((gts + rows_b - 1) // rows_b + 1)) if B else 0
    table = np.empty((max(cap, 1), 4), np.int64)
    want = 0 if ctas is None else max(1, int(ctas))
    bounds = np.empty(want + 1, np.int64)
    out = np.zeros(2, np.int64)  # total chunks, ranges
    n = N.call("pe_contract_blocks", dets.ctypes.data, gts.ctypes.data, pixels.ctypes.data,
               None if flags is None else flags.ctypes.data, B,
               CONTRACT_TMA_COST if tma_cost is None else float(tma_cost), want, table.ctypes.data, cap,
               bounds.ctypes.data, out.ctypes.data, out.ctypes.data + 8)
    table, total = table[:n], int(out[0])
    if ctas is None:
        return table, total
    return table, total, bounds[: int(out[1]) + 1]


def pass_bounds(pixels, dets, ctas, chunk=SEG_CHUNK):
    """ctas + 1 chunk indices splitting the fused pass into contiguous CTA ranges of about equal bytes.

    A chunk of image b costs its pixels x (8 + D_b) bytes (two int32 maps plus
    one byte per detection mask); chunks are numbered image by image.
    """
    pixels, dets = np.asarray(pixels, np.int64).reshape(-1), np.asarray(dets, np.int64).reshape(-1)
    chunks = -(-pixels // chunk)
    total = int(chunks.sum())
    ctas = max(1, min(int(ctas), total))
    if total == 0:
        return np.zeros(2, np.int64)
    first = np.cumsum(chunks) - chunks
    size = np.full(total, chunk, np.int64)
    live = chunks > 0
    size[(first + chunks - 1)[live]] = (pixels - chunk * (chunks - 1))[live]
    cost = np.cumsum(np.repeat(8 + dets, chunks) * size)
    inner = np.searchsorted(cost, cost[-1] * np.arange(1, ctas) / ctas, side="left") + 1
    return np.maximum.accumulate(np.concatenate(([0], np.minimum(inner, total), [total]))).astype(np.int64)


def aligned(ptr: int, stride_bytes: int = 0, to: int = 16) -> bool:
    return ptr % to == 0 and stride_bytes % to == 0


class Scratch:
    """Named device buffers reused across calls while their size fits."""

    def __init__(self, device):
        self.device = torch.device(device)
        self._buffers = {}
        self._views = {}  # name -> (numel, dtype, view) of the last request, reused while it repeats

    def get(self, name, numel, dtype, zero=False):
        numel = max(int(numel), 1)
        last = self._views.get(name)
        if last is not None and last[0] == numel and last[1] is dtype:
            view = last[2]
        else:
            buf = self._buffers.get(name)
            if buf is None or buf.numel() < numel or buf.dtype != dtype:
                buf = torch.empty(max(numel, int(1.25 * numel) if buf is not None else numel), dtype=dtype,
                                  device=self.device)
                self._buffers[name] = buf
            view = buf[:numel]
            self._views[name] = (numel, dtype, view)
        if zero:
            view.zero_()
        return view


def upload(host: np.ndarray, out: torch.Tensor) -> torch.Tensor:
    """Async host->device copy of an int64 array through pinned memory."""
    pinned = torch.empty(host.size, dtype=torch.int64, pin_memory=True)
    pinned.numpy()[:] = host.reshape(-1)
    out[: host.size].copy_(pinned, non_blocking=True)
    return out


# Per-image histogram bins of the batched passes are 32-bit counts, exact for any image below 2^32 pixels.
MAX_IMAGE_PIXELS = 2**32 - 1


def check_pixels(pixels):
    """Reject images whose pixel count the 32-bit per-image bins could not hold."""
    pixels = np.asarray(pixels, np.int64)
    if pixels.size and int(pixels.max()) > MAX_IMAGE_PIXELS:
        raise ValueError(f"an image has {int(pixels.max())} pixels; batched evaluation keeps 32-bit per-image "
                         f"counts and accepts at most {MAX_IMAGE_PIXELS} pixels per image")


class DescTable:
    """Descriptors [B, 16] followed by d_off [B+1], g_off [B+1], pair_off [B] (int64)."""

    def __init__(self, B):
        self.B = B
        self.desc = np.zeros((B, FIELDS), np.int64)

    def extra_offset(self):
        """int64 index at which ``finish``'s ``bounds`` array starts in the upload."""
        return self.B * FIELDS + 3 * self.B + 2

    def finish(self, scratch: Scratch, name="descs", bounds=None):
        """Upload descriptors, offsets and (optionally) the fused pass's CTA chunk bounds in one copy."""
        B = self.B
        d = self.desc
        check_pixels(d[:, PIXELS])
        d_off = np.concatenate(([0], np.cumsum(d[:, D])))
        g_off = np.concatenate(([0], np.cumsum(d[:, G])))
        extra = np.asarray(bounds, np.int64) if bounds is not None else np.zeros(0, np.int64)
        host = np.concatenate((d.reshape(-1), d_off, g_off, d[:, DPAIR_BEGIN], extra))
        buf = upload(host, scratch.get(name, host.size, torch.int64))
        self.device = buf
        self.descs = buf[: B * FIELDS]
        self.d_off = buf[B * FIELDS: B * FIELDS + B + 1]
        self.g_off = buf[B * FIELDS + B + 1: B * FIELDS + 2 * B + 2]
        self.pair_off = buf[B * FIELDS + 2 * B + 2: B * FIELDS + 3 * B + 2]
        start = self.extra_offset()
        self.bounds = buf[start: start + extra.size] if extra.size else None
        self.ctas = max(int(extra.size) - 1, 0)
        return self


class RecordStore:
    """Instance records between updates: scores f64, classes i32, ranks i32, flags i8 [n, 40]."""

    def __init__(self, device):
        self.device = torch.device(device)
        self.n = 0
        self._allocate(1024)

    def _allocate(self, capacity):
        self.capacity = capacity
        self.scores = torch.empty(capacity, dtype=torch.float64, device=self.device)
        self.classes = torch.empty(capacity, dtype=torch.int32, device=self.device)
        self.ranks = torch.empty(capacity, dtype=torch.int32, device=self.device)
        self.flags = torch.empty((capacity, CHAINS), dtype=torch.int8, device=self.device)

    def reserve(self, extra):
        need = self.n + extra
        if need <= self.capacity:
            return
        old = (self.scores, self.classes, self.ranks, self.flags)
        self._allocate(max(need, 2 * self.capacity))
        for new, prev in zip((self.scores, self.classes, self.ranks, self.flags), old):
            new[: self.n].copy_(prev[: self.n])

    def reset(self):
        self.n = 0

    def tail(self):
        """Views where the next records are written."""
        n = self.n
        return self.scores[n:], self.classes[n:], self.ranks[n:], self.flags[n:]
