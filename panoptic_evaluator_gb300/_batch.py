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


def contract_blocks(dets, gts, pixels, ctas=None):
    """Block table of pe_inst_contract: rows (image, first detection, first target, first chunk).

    Each image with pixels and at least one mask is covered by 127 x 63 tiles
    of ceil(pixels / 4096) chunks. With `ctas`, also returns ctas + 1 chunk
    bounds that give every CTA a contiguous range of about equal cost (mask
    rows x pixels). Returns (int64 [n, 4] array, total chunks[, bounds]).
    """
    rows, cost, chunk = [], [], 0
    for b, (d, g, hw) in enumerate(zip(dets, gts, pixels)):
        d, g, hw = int(d), int(g), int(hw)
        if hw <= 0 or (d == 0 and g == 0):
            continue
        n = -(-hw // CONTRACT_CHUNK)
        sizes = np.full(n, CONTRACT_CHUNK, np.int64)
        sizes[-1] = hw - CONTRACT_CHUNK * (n - 1)
        for m0 in range(0, max(d, 1), CONTRACT_ROWS[0]):
            for n0 in range(0, max(g, 1), CONTRACT_ROWS[1]):
                rows.append((b, m0, n0, chunk))
                active = min(CONTRACT_ROWS[0], d - m0) + min(CONTRACT_ROWS[1], g - n0)
                cost.append((active + 8) * sizes)  # +8: fixed work per stage (ones rows, MMA, barriers)
                chunk += n
    table = np.array(rows, np.int64).reshape(-1, 4)
    if ctas is None:
        return table, chunk
    ctas = max(1, min(int(ctas), chunk))
    if chunk == 0:
        return table, 0, np.zeros(2, np.int64)
    total = np.cumsum(np.concatenate(cost))
    targets = total[-1] * np.arange(1, ctas) / ctas
    inner = np.searchsorted(total, targets, side="left") + 1
    bounds = np.concatenate(([0], np.minimum(inner, chunk), [chunk])).astype(np.int64)
    bounds = np.maximum.accumulate(bounds)
    return table, chunk, bounds


def aligned(ptr: int, stride_bytes: int = 0, to: int = 16) -> bool:
    return ptr % to == 0 and stride_bytes % to == 0


class Scratch:
    """Named device buffers reused across calls while their size fits."""

    def __init__(self, device):
        self.device = torch.device(device)
        self._buffers = {}

    def get(self, name, numel, dtype, zero=False):
        numel = max(int(numel), 1)
        buf = self._buffers.get(name)
        if buf is None or buf.numel() < numel or buf.dtype != dtype:
            buf = torch.empty(max(numel, int(1.25 * numel) if buf is not None else numel), dtype=dtype,
                              device=self.device)
            self._buffers[name] = buf
        view = buf[:numel]
        if zero:
            view.zero_()
        return view


def upload(host: np.ndarray, out: torch.Tensor) -> torch.Tensor:
    """Async host->device copy of an int64 array through pinned memory."""
    pinned = torch.empty(host.size, dtype=torch.int64, pin_memory=True)
    pinned.numpy()[:] = host.reshape(-1)
    out[: host.size].copy_(pinned, non_blocking=True)
    return out


class DescTable:
    """Descriptors [B, 16] followed by d_off [B+1], g_off [B+1], pair_off [B] (int64)."""

    def __init__(self, B):
        self.B = B
        self.desc = np.zeros((B, FIELDS), np.int64)

    def finish(self, scratch: Scratch, name="descs"):
        B = self.B
        d = self.desc
        d_off = np.concatenate(([0], np.cumsum(d[:, D])))
        g_off = np.concatenate(([0], np.cumsum(d[:, G])))
        host = np.concatenate((d.reshape(-1), d_off, g_off, d[:, DPAIR_BEGIN]))
        buf = upload(host, scratch.get(name, host.size, torch.int64))
        self.device = buf
        self.descs = buf[: B * FIELDS]
        self.d_off = buf[B * FIELDS: B * FIELDS + B + 1]
        self.g_off = buf[B * FIELDS + B + 1: B * FIELDS + 2 * B + 2]
        self.pair_off = buf[B * FIELDS + 2 * B + 2: B * FIELDS + 3 * B + 2]
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


def pinned_copy(tensor: torch.Tensor) -> torch.Tensor:
    out = torch.empty(tensor.shape, dtype=tensor.dtype, pin_memory=True)
    out.copy_(tensor)
    return out


def native_ptr(tensor):
    return N.ptr(tensor)
