"""Reward serving: continuous batching of per-image PQ and generation-prefix requests on one GPU.

Requests carry host data in pinned memory. A scheduler thread admits queued
requests in arrival order while the batch being formed fits a free block of
the server's device arena (one allocation of ``memory_budget`` bytes made at
start-up: the loop itself never allocates device memory), groups them by kind
into batches and launches each batch on one of a few CUDA streams, so batches
that arrive while others run overlap on the device. A batch is a fixed number
of launches whatever its size:

* panoptic_quality requests (uneven image sizes): the fused pass over the
  slot maps (``pe_seg_pass``), per-image reward scoring (``pe_seg_score`` in
  reward mode) and the per-image mean-class PQ (``pe_reward_pq``), which also
  folds every request's statistics into dataset totals kept on the device;
* generation-prefix requests (uneven sizes, any checkpoints): ``pe_prefix``.

Every per-request quantity is computed inside that request's own CTAs with
fixed reduction orders, so a request's result is bit-identical whether it is
served alone or batched with others. Latency is measured from the request's
arrival timestamp to the moment its result is on the host.
"""

from __future__ import annotations

import collections
import gc
import statistics
import threading
import time
from collections.abc import Sequence
from concurrent.futures import Future
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _native as N
from . import prefix as PF
from ._batch import (CHUNK_BEGIN, FLAGS, G, MASK_STRIDE, PAIR_BEGIN, PIXELS, PRED, PSLOT_BEGIN, SEG_CHUNK,
                     SLOT_BEGIN, TARGET, FIELDS as SEG_FIELDS, P, check_pixels)

ALIGN = 256  # every buffer of a batch region starts on a 256-byte boundary
# Per-checkpoint fields copied back for prefix requests; the per-class tables only with full_results.
_PREFIX_KEYS = ("summaries", "counts", "miou", "itp", "ifp", "ifn", "precision", "recall")
_PREFIX_FULL_KEYS = ("tp", "fp", "fn", "sums", "confusion", "values")


def _admitted(job) -> bool:
    """Mark a queued request running (it can no longer be cancelled); False if it was cancelled.

    A request put back in the queue after admission is already running and stays admitted.
    """
    return job.future.running() or job.future.set_running_or_notify_cancel()


def _round(n, a=ALIGN):
    return (int(n) + a - 1) // a * a


def _pinned(nbytes):
    """Page-locked host bytes (plain host memory where no CUDA device exists, e.g. to build requests offline)."""
    return torch.empty(max(int(nbytes), 1), dtype=torch.uint8, pin_memory=torch.cuda.is_available())


class PanopticRequest:
    """One image for ``panoptic_quality``: prediction and target slot maps with their metadata."""

    kind = "panoptic"

    def __init__(self, pred, pred_classes, target, target_classes, crowd=None):
        target = np.ascontiguousarray(target, np.int32)
        pred = np.ascontiguousarray(pred, np.int32)
        if target.shape != pred.shape or target.ndim != 2 or target.size == 0:
            raise ValueError("prediction and target must be non-empty H x W maps of the same shape")
        self.hw = int(target.size)
        self.shape = target.shape
        self.target_classes = np.ascontiguousarray(target_classes, np.int32).reshape(-1)
        self.pred_classes = np.ascontiguousarray(pred_classes, np.int32).reshape(-1)
        if not len(self.target_classes) or not len(self.pred_classes):
            raise ValueError("slot 0 (void) must be present in both class tables")
        self.crowd = (np.zeros(len(self.target_classes), np.uint8) if crowd is None
                      else np.ascontiguousarray(crowd, np.uint8).reshape(-1))
        if len(self.crowd) != len(self.target_classes):
            raise ValueError("crowd needs one flag per target slot")
        self.span = _round(4 * self.hw)
        self.blob = _pinned(2 * self.span)  # [target | prediction], each 256-byte aligned
        view = self.blob.numpy()
        view[: 4 * self.hw] = target.reshape(-1).view(np.uint8)
        view[self.span: self.span + 4 * self.hw] = pred.reshape(-1).view(np.uint8)
        self.G, self.P = len(self.target_classes), len(self.pred_classes)
        self.chunks = -(-self.hw // SEG_CHUNK)


class PrefixRequest:
    """One generation-ordered mask sequence for ``segmentation_prefixes``."""

    kind = "prefix"

    def __init__(self, masks, classes, target, target_classes, crowd=None, checkpoints=None):
        target = np.ascontiguousarray(target, np.int32)
        masks = np.ascontiguousarray(masks, bool)
        if masks.ndim != 3 or masks.shape[1:] != target.shape or target.size == 0:
            raise ValueError("masks must be N x H x W with the target's (non-empty) H x W")
        self.n = int(masks.shape[0])
        self.hw = int(target.size)
        self.shape = target.shape
        self.classes = np.ascontiguousarray(classes, np.int32).reshape(-1)
        self.target_classes = np.ascontiguousarray(target_classes, np.int32).reshape(-1)
        if len(self.classes) != self.n or not len(self.target_classes):
            raise ValueError("one class per mask and a target class table with slot 0 are required")
        self.crowd = (np.zeros(len(self.target_classes), np.uint8) if crowd is None
                      else np.ascontiguousarray(crowd, np.uint8).reshape(-1))
        self.points = list(checkpoints) if checkpoints is not None else (list(range(1, self.n + 1)) if self.n else [0])
        if (not self.points or any(k < 0 or k > self.n for k in self.points)
                or any(a >= b for a, b in zip(self.points, self.points[1:]))):
            raise ValueError("checkpoints must be strictly increasing values in 0..N")
        self.pitch = _round(self.hw, 128)
        self.span = _round(4 * self.hw)
        self.blob = _pinned(self.span + self.n * self.pitch)  # [target | masks, rows padded to 128 bytes]
        view = self.blob.numpy()
        view[: 4 * self.hw] = target.reshape(-1).view(np.uint8)
        if self.n:
            rows = view[self.span: self.span + self.n * self.pitch].reshape(self.n, self.pitch)
            rows[:, : self.hw] = masks.reshape(self.n, self.hw).view(np.uint8)
            rows[:, self.hw:] = 0
        self.G = len(self.target_classes)
        self.steps = np.full(self.n + 1, -1, np.int32)  # checkpoint index at each prefix length
        for index, k in enumerate(self.points):
            self.steps[k] = index
        self.chunks = -(-self.hw // PF.CHUNK)


class PrefixSnapshots(Sequence):
    """The checkpoint snapshots of one prefix request, as the reference's per-checkpoint dicts.

    Backed by one numpy array per field (rows = this request's checkpoints);
    snapshot i is built as a dict when it is read. A response therefore holds a
    few untracked arrays instead of nested dicts, which keeps the cyclic
    garbage collector's work small while many responses are alive.
    """

    __slots__ = ("points", "fields", "thresholds")

    def __init__(self, points, fields, thresholds):
        self.points, self.fields, self.thresholds = tuple(points), fields, tuple(thresholds)

    def __len__(self):
        return len(self.points)

    def __getitem__(self, i):
        if isinstance(i, slice):
            return [self[j] for j in range(*i.indices(len(self)))]
        if i < 0:
            i += len(self)
        if not 0 <= i < len(self):
            raise IndexError(i)
        f = self.fields
        s, n = f["summaries"][i], f["counts"][i]
        snap = {name: dict(pq=float(s[g, 0]), sq=float(s[g, 1]), rq=float(s[g, 2]), n=int(n[g]))
                for g, name in enumerate(("All", "Things", "Stuff"))}
        snap.update(prefix=self.points[i], miou=float(f["miou"][i]),
                    instance=dict(iou_thresholds=np.array(self.thresholds), tp=f["itp"][i], fp=f["ifp"][i],
                                  fn=f["ifn"][i], precision=f["precision"][i], recall=f["recall"][i]))
        if "values" in f:
            v = f["values"][i]
            snap.update(tp=f["tp"][i], fp=f["fp"][i], fn=f["fn"][i], iou_sum=f["sums"][i], confusion=f["confusion"][i],
                        per_class={name: v[g] for g, name in enumerate(("pq", "sq", "rq", "iou"))})
        return snap


@dataclass
class Response:
    """Result of one request: ``values`` holds numpy arrays, ``latency_ms`` is arrival -> result on host."""

    kind: str
    values: dict
    latency_ms: float
    batch_size: int


@dataclass
class _Job:
    request: object
    future: Future
    arrival: float


@dataclass
class _Batch:
    kind: str
    jobs: list
    stream: torch.cuda.Stream
    event: torch.cuda.Event
    offset: int
    nbytes: int
    keep: list = field(default_factory=list)
    host: dict = field(default_factory=dict)
    rows: object = None
    begin: object = None  # timing event before the first copy (tracing only)
    host_offset: int = -1  # pinned staging region (metadata in, results out); -1: own allocation
    host_nbytes: int = 0
    t_admit: float = 0.0
    t_launched: float = 0.0


class _Arena:
    """First-fit allocator of aligned byte ranges inside one buffer (device memory, or pinned host memory)."""

    def __init__(self, nbytes, device, pinned=False):
        self.nbytes = int(nbytes)
        self.buffer = torch.empty(self.nbytes, dtype=torch.uint8, device=device, pin_memory=pinned)
        self.free = [(0, self.nbytes)]  # sorted, coalesced (offset, size)
        self.used = 0

    def allocate(self, size):
        size = _round(size)
        for i, (off, n) in enumerate(self.free):
            if n >= size:
                if n == size:
                    del self.free[i]
                else:
                    self.free[i] = (off + size, n - size)
                self.used += size
                return off
        return None

    def release(self, off, size):
        size = _round(size)
        self.used -= size
        self.free.append((off, size))
        self.free.sort()
        merged = []
        for o, n in self.free:
            if merged and merged[-1][0] + merged[-1][1] == o:
                merged[-1] = (merged[-1][0], merged[-1][1] + n)
            else:
                merged.append((o, n))
        self.free = merged

    def largest(self):
        return max((n for _, n in self.free), default=0)


class _Layout:
    """Named, 256-byte-aligned sub-buffers of one batch region."""

    def __init__(self):
        self.parts = {}
        self.size = 0

    def add(self, name, nbytes):
        off = _round(self.size)
        self.parts[name] = (off, int(nbytes))
        self.size = off + int(nbytes)

    def view(self, region, name, dtype, shape=None):
        off, nbytes = self.parts[name]
        itemsize = torch.empty((), dtype=dtype).element_size()
        count = nbytes // itemsize
        t = region[off: off + count * itemsize].view(dtype)
        return t.reshape(shape) if shape is not None else t


class RewardServer:
    """Continuous-batching reward server on one GPU (see the module docstring).

    ``memory_budget`` bytes of device memory are reserved at construction and
    every batch (inputs, scratch, outputs) is carved from them; ``max_batch``
    and ``max_batch_bytes`` bound one batch; ``streams`` batches may run at once.
    """

    def __init__(self, num_classes, *, isthing=None, iou_thresholds=(0.5, 0.75), device="cuda",
                 memory_budget=4 << 30, max_batch=64, max_batch_bytes=256 << 20, streams=4, validate=False,
                 full_results=False, trace=False, host_staging=64 << 20):
        self.device = torch.device(device)
        if self.device.type != "cuda":
            raise ValueError("pe_gb300 evaluates on CUDA devices only")
        if self.device.index is None:
            self.device = torch.device("cuda", torch.cuda.current_device())
        self.num_classes = num_classes
        self.validate = validate
        self.full_results = full_results
        self.max_batch = max_batch
        self.max_batch_bytes = int(max_batch_bytes)
        self.memory_budget = int(memory_budget)
        self.thresholds = tuple(float(t) for t in iou_thresholds)
        with torch.cuda.device(self.device):
            self.isthing = torch.tensor(isthing if isthing is not None else [True] * num_classes, dtype=torch.bool,
                                        device=self.device)
            self._things_u8 = self.isthing.to(torch.uint8)
            self._thr = torch.tensor(self.thresholds, dtype=torch.float64, device=self.device)
            self._streams = [torch.cuda.Stream(self.device) for _ in range(streams)]
            C = num_classes
            # Dataset totals of every served panoptic request, kept on the device.
            self.totals = dict(tp=torch.zeros(C, dtype=torch.int64, device=self.device),
                               fp=torch.zeros(C, dtype=torch.int64, device=self.device),
                               fn=torch.zeros(C, dtype=torch.int64, device=self.device),
                               iou_sum=torch.zeros(C, dtype=torch.float64, device=self.device))
            self._arena = _Arena(self.memory_budget, self.device)
        # Pinned host memory for every batch's metadata upload and result read-back, reserved once:
        # page-locking fresh host memory per batch costs milliseconds.
        self._host = _Arena(host_staging, "cpu", pinned=True)
        self._lock = threading.Condition()
        self._pending = collections.deque()
        self._in_flight = []
        self.peak_in_flight_bytes = 0
        self.batches = 0
        # With trace=True, one dict per completed batch: kind, size, queue wait of its oldest request,
        # host launch time, device time (copies + kernels + read-back) and completion-to-host delay (ms).
        self.trace = [] if trace else None
        self._stop = False
        self._thread = None
        self._finisher = None

    # ---- sizes ---------------------------------------------------------------
    def footprint(self, request):
        """Device bytes a request adds to its batch (inputs, scratch and outputs, with alignment slack)."""
        C, T = self.num_classes, len(self.thresholds)
        if request.kind == "panoptic":
            g, p = request.G, request.P
            return (_round(request.blob.numel()) + 8 * SEG_FIELDS + 9 * g + 4 * p + 4 * g * p + 8 * (g + p)
                    + 4 * g + 32 * C + 8 + 64)
        n, g, q = request.n, request.G, len(request.points)
        per_row = 8 * C * 8 + 8 * C * (C + 1) + 40 * T * C + 8 * 9 + 8 * 3 + 8
        return (_round(request.blob.numel()) + 8 * PF.FIELDS + 4 * (n + 1) + 4 * n + 5 * g + q * per_row
                + 4 * g + 4 * n * g + 4 * q * g * (n + 1) + 8 * T * C + 64)

    _OVERHEAD = 24 * ALIGN  # alignment of the batch's named buffers

    # ---- client side -------------------------------------------------------
    def submit(self, request, arrival=None) -> Future:
        """Queue a request; the future resolves to a Response. `arrival` defaults to now.

        A request whose future is cancelled before it is admitted is dropped; once admitted
        (the future is running) it cannot be cancelled.
        """
        future = Future()
        job = _Job(request, future, time.perf_counter() if arrival is None else arrival)
        with self._lock:
            self._pending.append(job)
            self._lock.notify()
        return future

    def start(self):
        if self._thread is None:
            self._stop = False
            self._thread = threading.Thread(target=self._run, name="pe-reward-scheduler", daemon=True)
            self._finisher = threading.Thread(target=self._finish, name="pe-reward-completion", daemon=True)
            self._thread.start()
            self._finisher.start()
        return self

    def stop(self):
        """Serve everything queued, then stop the server threads."""
        with self._lock:
            self._stop = True
            self._lock.notify_all()
        for thread in (self._thread, self._finisher):
            if thread is not None:
                thread.join()
        self._thread = self._finisher = None

    def __enter__(self):
        return self.start()

    def __exit__(self, *exc):
        self.stop()

    # ---- scheduler -----------------------------------------------------------
    def _run(self):
        """Scheduler thread: admit and launch batches whenever requests and a stream are available."""
        torch.cuda.set_device(self.device)
        while True:
            self._launch()
            with self._lock:
                if self._stop and not self._pending and not self._in_flight:
                    return
                if not self._pending or len(self._in_flight) >= len(self._streams):
                    self._lock.wait(timeout=0.01)

    def _finish(self):
        """Completion thread: hand results to their futures as soon as a batch's work is done."""
        torch.cuda.set_device(self.device)
        while True:
            with self._lock:
                batches = list(self._in_flight)
                if self._stop and not self._pending and not batches and not (self._thread and
                                                                             self._thread.is_alive()):
                    return
            done = [b for b in batches if b.event.query()]
            if not done:
                time.sleep(0.00005)  # releases the interpreter; ~50-100 us detection granularity
                continue
            for batch in done:
                self._complete(batch)
            with self._lock:
                self._lock.notify_all()  # a stream and arena space are free again

    def _complete(self, batch):
        with self._lock:
            self._in_flight.remove(batch)
            self._arena.release(batch.offset, batch.nbytes)
        now = time.perf_counter()
        self._finalize(batch, now)
        if batch.host_offset >= 0:
            with self._lock:
                self._host.release(batch.host_offset, batch.host_nbytes)

    def _host_region(self, nbytes):
        """(offset, pinned uint8 view) for a batch's staging; offset -1 when the reserved area is full."""
        with self._lock:
            off = self._host.allocate(nbytes)
        if off is None:
            return -1, _pinned(nbytes)
        self._launch_host = (off, nbytes)  # released by _launch if the batch fails to launch
        return off, self._host.buffer[off: off + _round(nbytes)]

    def _finalize(self, batch, now):
        if self.trace is not None:
            device_ms = batch.begin.elapsed_time(batch.event)
            self.trace.append(dict(kind=batch.kind, size=len(batch.jobs),
                                   queue_ms=1000 * (batch.t_admit - min(j.arrival for j in batch.jobs)),
                                   launch_ms=1000 * (batch.t_launched - batch.t_admit), device_ms=device_ms,
                                   detect_ms=1000 * (now - batch.t_launched) - device_ms))
        code = int(batch.host["error"][0])
        for index, job in enumerate(batch.jobs):
            if code:
                job.future.set_exception(ValueError(f"invalid request in batch (error bits {code:#x})"))
                continue
            values = self._unpack(batch, index)
            job.future.set_result(Response(batch.kind, values, 1000 * (now - job.arrival), len(batch.jobs)))

    def _admit(self):
        """Next batch: requests of the head request's kind, in arrival order, that fit one free arena block.

        Returns (kind, jobs, bytes) or None. Requests of the other kind stay queued for the next batch.
        """
        with self._lock:
            if len(self._in_flight) >= len(self._streams):
                return None
            if any(job.future.cancelled() for job in self._pending):  # cancelled while queued: dropped
                self._pending = collections.deque(job for job in self._pending if not job.future.cancelled())
            while self._pending:
                job = self._pending[0]
                need = self.footprint(job.request)
                if _round(need + self._OVERHEAD) <= self._arena.nbytes:
                    break
                self._pending.popleft()
                if _admitted(job):
                    job.future.set_exception(ValueError(
                        f"request needs {need} bytes of device memory, above the {self._arena.nbytes}-byte budget"))
            if not self._pending:
                return None
            kind = self._pending[0].request.kind
            room = self._arena.largest()
            taken, kept = [], collections.deque()
            total, blobs, full = self._OVERHEAD, 0, False
            for job in self._pending:
                if full or job.request.kind != kind:
                    kept.append(job)
                    continue
                need = self.footprint(job.request)
                blob = _round(job.request.blob.numel())
                if taken and (len(taken) >= self.max_batch or blobs + blob > self.max_batch_bytes):
                    full = True
                elif _round(total + need) > room:
                    full = True
                if full:
                    kept.append(job)
                    continue
                taken.append(job)
                total += need
                blobs += blob
            # Admitted requests can no longer be cancelled; one cancelled since the filter above is dropped.
            taken = [job for job in taken if _admitted(job)]
            self._pending = kept
            if not taken:
                return None
        return kind, taken, _round(total)

    def _launch(self):
        launched = False
        while True:
            admitted = self._admit()
            if admitted is None:
                return launched
            kind, jobs, nbytes = admitted
            with self._lock:
                offset = self._arena.allocate(nbytes)
            if offset is None:  # cannot happen after the size check; requeue defensively
                with self._lock:
                    self._pending.extendleft(reversed(jobs))
                return launched
            with self._lock:
                free = [s for s in self._streams if all(b.stream is not s for b in self._in_flight)]
            stream = free[0] if free else self._streams[self.batches % len(self._streams)]
            region = self._arena.buffer[offset: offset + nbytes]
            t_admit = time.perf_counter()
            begin = None
            if self.trace is not None:
                begin = torch.cuda.Event(enable_timing=True)
                begin.record(stream)
            self._launch_host = None
            try:
                launch = self._launch_panoptic if kind == "panoptic" else self._launch_prefix
                batch = launch(jobs, stream, region)
            except Exception as error:  # report on every request of the batch
                with self._lock:
                    self._arena.release(offset, nbytes)
                    if self._launch_host is not None:
                        self._host.release(*self._launch_host)
                for job in jobs:
                    job.future.set_exception(error)
                continue
            batch.offset, batch.nbytes = offset, nbytes
            batch.begin, batch.t_admit, batch.t_launched = begin, t_admit, time.perf_counter()
            with self._lock:
                self._in_flight.append(batch)
                self.peak_in_flight_bytes = max(self.peak_in_flight_bytes, self._arena.used)
                self.batches += 1
            launched = True

    # ---- batches -------------------------------------------------------------
    @staticmethod
    def _upload_blobs(reqs, region, layout):
        base = layout.parts["blobs"][0]
        offsets, off = [], base
        for r in reqs:
            n = r.blob.numel()
            region[off: off + n].copy_(r.blob, non_blocking=True)
            offsets.append(off)
            off += _round(n)
        return np.array(offsets, np.int64)

    @staticmethod
    def _meta_span(layout, names):
        first = min(layout.parts[name][0] for name in names)
        return first, max(layout.parts[name][0] + layout.parts[name][1] for name in names) - first

    @staticmethod
    def _upload_meta(region, layout, parts, host):
        """One pinned staging view for every small metadata array (named parts of the layout), one copy."""
        first = min(layout.parts[name][0] for name, _ in parts)
        last = max(layout.parts[name][0] + layout.parts[name][1] for name, _ in parts)
        view = host.numpy()
        for name, array in parts:
            off = layout.parts[name][0] - first
            raw = np.ascontiguousarray(array).reshape(-1).view(np.uint8)
            view[off: off + raw.size] = raw
        region[first: last].copy_(host[: last - first], non_blocking=True)
        return host

    @staticmethod
    def _results(fields):
        """Offsets of (name, dtype, shape) fields packed 8-byte aligned into one block, and its size."""
        offsets, size = {}, 0
        for name, dtype, shape in fields:
            offsets[name] = (size, dtype, shape)
            size += (int(np.prod(shape)) * np.dtype(dtype).itemsize + 7) // 8 * 8
        return offsets, size

    @staticmethod
    def _read_back(region, layout, block, fields, size, host):
        """Copy the result block to the pinned view (one copy); numpy views of its fields."""
        off = layout.parts[block][0]
        host = host[:size]
        host.copy_(region[off: off + size], non_blocking=True)
        raw = host.numpy()
        views = {name: raw[o: o + int(np.prod(shape)) * np.dtype(dt).itemsize].view(dt).reshape(shape)
                 for name, (o, dt, shape) in fields.items()}
        return host, views

    def _launch_panoptic(self, jobs, stream, region):
        reqs = [j.request for j in jobs]
        B, C = len(reqs), self.num_classes
        Gs = np.array([r.G for r in reqs], np.int64)
        Ps = np.array([r.P for r in reqs], np.int64)
        hw = np.array([r.hw for r in reqs], np.int64)
        chunks = np.array([r.chunks for r in reqs], np.int64)
        pan = Gs * Ps
        fields, result_bytes = self._results([("pq", np.float64, (B,)), ("error", np.int32, (1,))])
        L = _Layout()
        L.add("blobs", sum(_round(r.blob.numel()) for r in reqs))
        L.add("descs", 8 * B * SEG_FIELDS)
        L.add("gc", 4 * int(Gs.sum()))
        L.add("pc", 4 * int(Ps.sum()))
        L.add("crowd", int(Gs.sum()))
        L.add("result", result_bytes)  # right after the metadata: one upload also zeroes the error word
        L.add("pairs", 4 * max(int(pan.sum()), 1))
        L.add("areas", 8 * int((Gs + Ps).sum()))
        L.add("matched", 4 * int(Gs.sum()))
        L.add("stats", 8 * 4 * B * C)  # tp, fp, fn rows, then iou sums: zeroed together
        L.add("schedule", 8)  # chunk counter of the fused pass
        base = region.data_ptr()
        ptr = lambda name, extra=0: base + L.parts[name][0] + extra  # noqa: E731
        with torch.cuda.stream(stream):
            offsets = self._upload_blobs(reqs, region, L)
            d = np.zeros((B, SEG_FIELDS), np.int64)
            d[:, TARGET] = base + offsets
            d[:, PRED] = base + offsets + np.array([r.span for r in reqs], np.int64)
            check_pixels(hw)
            d[:, PIXELS] = hw
            d[:, MASK_STRIDE] = 16
            d[:, CHUNK_BEGIN] = np.cumsum(chunks) - chunks
            d[:, SLOT_BEGIN] = np.cumsum(Gs) - Gs
            d[:, PSLOT_BEGIN] = np.cumsum(Ps) - Ps
            d[:, PAIR_BEGIN] = np.cumsum(pan) - pan
            d[:, G] = Gs
            d[:, P] = Ps
            d[:, FLAGS] = 3
            _, meta_bytes = self._meta_span(L, ("descs", "gc", "pc", "crowd", "result"))
            host_off, staging = self._host_region(_round(meta_bytes) + _round(result_bytes))
            host_meta = self._upload_meta(region, L, [
                ("descs", d), ("gc", np.concatenate([r.target_classes for r in reqs])),
                ("pc", np.concatenate([r.pred_classes for r in reqs])),
                ("crowd", np.concatenate([r.crowd for r in reqs])),
                ("result", np.zeros(result_bytes, np.uint8))], staging[: _round(meta_bytes)])  # zeroes the error word
            so = L.parts["stats"][0]
            region[so: so + 32 * B * C].zero_()
            tp, fp, fn, sums = (ptr("stats", 8 * B * C * k) for k in range(4))
            error = ptr("result", fields["error"][0])
            h = N.stream_handle(self.device)
            N.call("pe_seg_pass", ptr("descs"), B, int(chunks.sum()), None, ptr("pairs"), int(pan.sum()), None, 0,
                   int(pan.max()), 0, 1, None, 0, ptr("schedule"), error, h)
            N.call("pe_seg_score", ptr("descs"), B, int(Ps.max()), int(pan.max()), ptr("pairs"), None, ptr("gc"),
                   ptr("pc"),
                   ptr("crowd"), ptr("areas"), ptr("matched"), tp, fp, fn, sums, None, C, N.ptr(self._things_u8),
                   None, None, None, None, None, None, None, int(self.validate), 1, None, error, h)
            t = self.totals
            N.call("pe_reward_pq", tp, fp, fn, sums, B, C, ptr("result", fields["pq"][0]), N.ptr(t["tp"]),
                   N.ptr(t["fp"]), N.ptr(t["fn"]), N.ptr(t["iou_sum"]), h)
            host, views = self._read_back(region, L, "result", fields, result_bytes, staging[_round(meta_bytes):])
            event = torch.cuda.Event(enable_timing=self.trace is not None)
            event.record(stream)
        batch = _Batch("panoptic", jobs, stream, event, 0, 0)
        batch.host_offset, batch.host_nbytes = host_off, _round(meta_bytes) + _round(result_bytes)
        batch.keep = [host_meta, host]
        batch.host = views
        return batch

    def _launch_prefix(self, jobs, stream, region):
        reqs = [j.request for j in jobs]
        B, C, T = len(reqs), self.num_classes, len(self.thresholds)
        n = np.array([r.n for r in reqs], np.int64)
        Gs = np.array([r.G for r in reqs], np.int64)
        q = np.array([len(r.points) for r in reqs], np.int64)
        hw = np.array([r.hw for r in reqs], np.int64)
        chunks = np.array([r.chunks for r in reqs], np.int64)
        cells = q * Gs * (n + 1)
        R = int(q.sum())
        shapes = dict(summaries=(R, 3, 3), counts=(R, 3), miou=(R,), itp=(R, T, C), ifp=(R, T, C), ifn=(R, T, C),
                      precision=(R, T, C), recall=(R, T, C), tp=(R, C), fp=(R, C), fn=(R, C), sums=(R, C),
                      confusion=(R, C, C + 1), values=(R, 4, C))
        doubles = {"sums", "precision", "recall", "values", "summaries", "miou"}
        keys = _PREFIX_KEYS + (_PREFIX_FULL_KEYS if self.full_results else ())
        fields, result_bytes = self._results(
            [(k, np.float64 if k in doubles else np.int64, shapes[k]) for k in keys] + [("error", np.int32, (1,))])
        L = _Layout()
        L.add("blobs", sum(_round(r.blob.numel()) for r in reqs))
        L.add("descs", 8 * B * PF.FIELDS)
        L.add("steps", 4 * int((n + 1).sum()))
        L.add("classes", 4 * max(int(n.sum()), 1))
        L.add("gc", 4 * int(Gs.sum()))
        L.add("crowd", int(Gs.sum()))
        L.add("result", result_bytes)
        for key in shapes:
            if key not in fields:
                L.add("out." + key, 8 * int(np.prod(shapes[key])))
        L.add("ga", 4 * int(Gs.sum()))
        L.add("raw", 4 * max(int((n * Gs).sum()), 1))
        L.add("pairs", 4 * max(int(cells.sum()), 1))
        L.add("counters", 4 * B * T * C * 2)
        L.add("schedule", 8)  # chunk counter of the owner pass
        base = region.data_ptr()
        ptr = lambda name: base + L.parts[name][0]  # noqa: E731
        out = {k: ptr("result") + fields[k][0] if k in fields else ptr("out." + k) for k in shapes}
        with torch.cuda.stream(stream):
            offsets = self._upload_blobs(reqs, region, L)
            d = np.zeros((B, PF.FIELDS), np.int64)
            d[:, PF.TARGET] = base + offsets
            d[:, PF.MASKS] = base + offsets + np.array([r.span for r in reqs], np.int64)
            check_pixels(hw)
            d[:, PF.PIXELS] = hw
            d[:, PF.STRIDE] = [r.pitch for r in reqs]
            d[:, PF.CHUNK_BEGIN] = np.cumsum(chunks) - chunks
            d[:, PF.NMASK] = n
            d[:, PF.NSLOT] = Gs
            d[:, PF.DET_BEGIN] = np.cumsum(n) - n
            d[:, PF.SLOT_BEGIN] = np.cumsum(Gs) - Gs
            d[:, PF.Q_BEGIN] = np.cumsum(q) - q
            d[:, PF.NQ] = q
            d[:, PF.PAIR_BEGIN] = np.cumsum(cells) - cells
            d[:, PF.RAW_BEGIN] = np.cumsum(n * Gs) - n * Gs
            d[:, PF.FLAGS] = 3
            d[:, PF.STEP_BEGIN] = np.cumsum(n + 1) - (n + 1)
            d[:, PF.COUNT_BEGIN] = np.arange(B) * T * C * 2
            _, meta_bytes = self._meta_span(L, ("descs", "steps", "classes", "gc", "crowd"))
            host_off, staging = self._host_region(_round(meta_bytes) + _round(result_bytes))
            host_meta = self._upload_meta(region, L, [
                ("descs", d), ("steps", np.concatenate([r.steps for r in reqs])),
                ("classes", np.concatenate([r.classes for r in reqs]) if n.sum() else np.zeros(1, np.int32)),
                ("gc", np.concatenate([r.target_classes for r in reqs])),
                ("crowd", np.concatenate([r.crowd for r in reqs]))], staging[: _round(meta_bytes)])
            N.call("pe_prefix", ptr("descs"), B, int(chunks.sum()), R, int(Gs.max()), int(n.max()) + 1,
                   int((Gs * (n + 1)).max()), ptr("steps"), ptr("classes"), ptr("gc"), ptr("crowd"),
                   N.ptr(self._things_u8), N.ptr(self._thr), T, C, ptr("ga"), int(Gs.sum()), ptr("raw"),
                   int((n * Gs).sum()), ptr("pairs"), int(cells.sum()), ptr("counters"), B * T * C * 2,
                   *[out[k] for k in ("tp", "fp", "fn", "sums", "confusion", "itp", "ifp", "ifn", "precision",
                                      "recall", "values", "summaries", "counts", "miou")],
                   int(self.validate), 1, ptr("schedule"), ptr("result") + fields["error"][0],
                   N.stream_handle(self.device))
            host, views = self._read_back(region, L, "result", fields, result_bytes, staging[_round(meta_bytes):])
            event = torch.cuda.Event(enable_timing=self.trace is not None)
            event.record(stream)
        batch = _Batch("prefix", jobs, stream, event, 0, 0)
        batch.host_offset, batch.host_nbytes = host_off, _round(meta_bytes) + _round(result_bytes)
        batch.keep = [host_meta, host]
        batch.host = views
        batch.rows = d[:, PF.Q_BEGIN].copy()
        return batch

    def _unpack(self, batch, index):
        if batch.kind == "panoptic":
            return dict(pq=float(batch.host["pq"][index]))
        req = batch.jobs[index].request
        first = int(batch.rows[index])
        rows = slice(first, first + len(req.points))
        # One copy of this request's rows per field (the pinned staging is reused by later batches).
        fields = {key: value[rows].copy() for key, value in batch.host.items() if key != "error"}
        return dict(snapshots=PrefixSnapshots(req.points, fields, self.thresholds))


def serve(server: RewardServer, requests, arrivals, *, pause_gc=False, freeze_gc=False):
    """Submit `requests` at `arrivals` (seconds from now, ascending) and wait for all.

    Returns (responses, summary) where summary has throughput and p50/p99 latency.
    By default the interpreter's cyclic garbage collector runs as it does for
    any caller of the server, and its pauses are part of the latencies. A full
    (generation 2) collection walks every tracked object of the process, so its
    pause grows with everything the application holds, not with the server.
    ``freeze_gc`` moves the objects that exist when the run starts out of the
    collector's scans (``gc.freeze()``; undone afterwards): collections still
    run, over what the run allocates. ``pause_gc`` instead disables the
    collector for the run (reference counting still frees memory).
    """
    server.start()
    paused = pause_gc and gc.isenabled()
    frozen = freeze_gc and not paused
    if paused:
        gc.collect()
        gc.disable()
    if frozen:
        gc.collect()
        gc.freeze()
    try:
        t0 = time.perf_counter()
        futures = []
        for request, at in zip(requests, arrivals):
            target = t0 + at
            wait = target - time.perf_counter()
            if wait > 0:
                time.sleep(wait)  # sleeping (not spinning) leaves the interpreter to the server threads
            futures.append(server.submit(request, arrival=target))
        responses = [f.result() for f in futures]
        wall = time.perf_counter() - t0
    finally:
        if paused:
            gc.enable()
        if frozen:
            gc.unfreeze()
    lat = sorted(r.latency_ms for r in responses)
    pick = lambda p: lat[min(len(lat) - 1, int(round(p * (len(lat) - 1))))]  # noqa: E731
    summary = dict(requests=len(responses), wall_s=wall, throughput=len(responses) / wall,
                   p50_ms=pick(0.50), p99_ms=pick(0.99), mean_ms=statistics.fmean(lat),
                   batches=server.batches, peak_in_flight_bytes=server.peak_in_flight_bytes,
                   mean_batch=statistics.fmean(r.batch_size for r in responses), gc_paused=bool(paused),
                   gc_frozen=bool(frozen), max_ms=lat[-1])
    return responses, summary
