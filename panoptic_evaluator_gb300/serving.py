"""Reward serving: continuous batching of per-image PQ and generation-prefix requests on one GPU.

Requests carry host data (pinned). A scheduler thread admits queued requests
in arrival order while their device footprint fits the HBM budget, groups the
admitted requests by kind into batches and launches each batch on one of a
few CUDA streams, so batches that arrive while others run overlap on the
device. A batch is a fixed number of launches regardless of its size:

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
import statistics
import threading
import time
from concurrent.futures import Future
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _native as N
from . import prefix as PF
from ._batch import (CHUNK_BEGIN, FLAGS, G, MASK_STRIDE, PAIR_BEGIN, PIXELS, PRED, PSLOT_BEGIN, SEG_CHUNK,
                     SLOT_BEGIN, TARGET, FIELDS as SEG_FIELDS, P)

ALIGN = 128
# Per-checkpoint fields copied back for prefix requests; the per-class tables only with full_results.
_PREFIX_KEYS = ("summaries", "counts", "miou", "itp", "ifp", "ifn", "precision", "recall")
_PREFIX_FULL_KEYS = ("tp", "fp", "fn", "sums", "confusion", "values")


def _round(n, a=ALIGN):
    return (n + a - 1) // a * a


def _pinned(nbytes):
    """Page-locked host bytes (plain host memory where no CUDA device exists, e.g. to build requests offline)."""
    return torch.empty(max(int(nbytes), 1), dtype=torch.uint8, pin_memory=torch.cuda.is_available())


class PanopticRequest:
    """One image for ``panoptic_quality``: prediction and target slot maps with their metadata."""

    kind = "panoptic"

    def __init__(self, pred, pred_classes, target, target_classes, crowd=None):
        target = np.ascontiguousarray(target, np.int32)
        pred = np.ascontiguousarray(pred, np.int32)
        if target.shape != pred.shape or target.ndim != 2:
            raise ValueError("prediction and target must be H x W maps of the same shape")
        self.hw = int(target.size)
        self.shape = target.shape
        self.target_classes = np.ascontiguousarray(target_classes, np.int32)
        self.pred_classes = np.ascontiguousarray(pred_classes, np.int32)
        self.crowd = (np.zeros(len(self.target_classes), np.uint8) if crowd is None
                      else np.ascontiguousarray(crowd, np.uint8))
        span = _round(4 * self.hw)
        self.blob = _pinned(2 * span)  # [target | prediction], each 128-byte aligned
        view = self.blob.numpy()
        view[: 4 * self.hw] = target.reshape(-1).view(np.uint8)
        view[span: span + 4 * self.hw] = pred.reshape(-1).view(np.uint8)
        self.span = span
        G_, P_ = len(self.target_classes), len(self.pred_classes)
        # Device bytes without the per-class outputs: maps, pair histogram, areas, metadata.
        self.nbytes = 2 * span + 4 * G_ * P_ + 8 * (G_ + P_) + 16 * G_ + 4 * P_ + 256


class PrefixRequest:
    """One generation-ordered mask sequence for ``segmentation_prefixes``."""

    kind = "prefix"

    def __init__(self, masks, classes, target, target_classes, crowd=None, checkpoints=None):
        target = np.ascontiguousarray(target, np.int32)
        masks = np.ascontiguousarray(masks, bool)
        if masks.ndim != 3 or masks.shape[1:] != target.shape:
            raise ValueError("masks must be N x H x W with the target's H x W")
        self.n = int(masks.shape[0])
        self.hw = int(target.size)
        self.shape = target.shape
        self.classes = np.ascontiguousarray(classes, np.int32)
        self.target_classes = np.ascontiguousarray(target_classes, np.int32)
        self.crowd = (np.zeros(len(self.target_classes), np.uint8) if crowd is None
                      else np.ascontiguousarray(crowd, np.uint8))
        self.points = list(checkpoints) if checkpoints is not None else (list(range(1, self.n + 1)) if self.n else [0])
        if any(k < 0 or k > self.n for k in self.points) or any(a >= b for a, b in zip(self.points, self.points[1:])):
            raise ValueError("checkpoints must be strictly increasing values in 0..N")
        self.pitch = _round(self.hw)
        span = _round(4 * self.hw)
        self.blob = _pinned(span + self.n * self.pitch)  # [target | masks, rows padded to 128 bytes]
        view = self.blob.numpy()
        view[: 4 * self.hw] = target.reshape(-1).view(np.uint8)
        if self.n:
            rows = view[span: span + self.n * self.pitch].reshape(self.n, self.pitch)
            rows[:, : self.hw] = masks.reshape(self.n, self.hw).view(np.uint8)
            rows[:, self.hw:] = 0
        self.span = span
        G_, Q = len(self.target_classes), len(self.points)
        # Device bytes without the per-checkpoint outputs: target, masks, histograms, metadata.
        self.nbytes = span + self.n * self.pitch + 4 * (Q * G_ * (self.n + 1) + self.n * G_ + 2 * G_ + 2 * self.n) + 256


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
    nbytes: int
    keep: list = field(default_factory=list)
    host: dict = field(default_factory=dict)
    layout: object = None


class RewardServer:
    """Continuous-batching reward server on one GPU (see the module docstring)."""

    def __init__(self, num_classes, *, isthing=None, iou_thresholds=(0.5, 0.75), device="cuda",
                 memory_budget=4 << 30, max_batch=64, streams=4, validate=False, full_results=False):
        self.device = torch.device(device)
        if self.device.type != "cuda":
            raise ValueError("pe_gb300 evaluates on CUDA devices only")
        if self.device.index is None:
            self.device = torch.device("cuda", torch.cuda.current_device())
        self.num_classes = num_classes
        self.validate = validate
        self.full_results = full_results
        self.max_batch = max_batch
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
        self._lock = threading.Condition()
        self._pending = collections.deque()
        self._in_flight = []
        self._in_flight_bytes = 0
        self.peak_in_flight_bytes = 0
        self.batches = 0
        self._stop = False
        self._thread = None

    def footprint(self, request):
        """Device bytes a request holds while in flight (inputs, scratch and outputs)."""
        C, T = self.num_classes, len(self.thresholds)
        if request.kind == "panoptic":
            return request.nbytes + 32 * C + 8
        rows = len(request.points)
        per_row = 8 * C * (4 + 4) + 8 * C * (C + 1) + 40 * T * C + 8 * 9 + 8 * 3 + 8
        return request.nbytes + rows * per_row + 8 * T * C

    # ---- client side -------------------------------------------------------
    def submit(self, request, arrival=None) -> Future:
        """Queue a request; the future resolves to a Response. `arrival` defaults to now."""
        future = Future()
        job = _Job(request, future, time.perf_counter() if arrival is None else arrival)
        with self._lock:
            self._pending.append(job)
            self._lock.notify()
        return future

    def start(self):
        if self._thread is None:
            self._stop = False
            self._thread = threading.Thread(target=self._run, name="pe-reward-server", daemon=True)
            self._thread.start()
        return self

    def stop(self):
        """Serve everything queued, then stop the scheduler thread."""
        with self._lock:
            self._stop = True
            self._lock.notify()
        if self._thread is not None:
            self._thread.join()
            self._thread = None

    def __enter__(self):
        return self.start()

    def __exit__(self, *exc):
        self.stop()

    # ---- scheduler -----------------------------------------------------------
    def _run(self):
        torch.cuda.set_device(self.device)
        while True:
            self._poll()
            launched = self._launch()
            with self._lock:
                if self._stop and not self._pending and not self._in_flight:
                    return
                if not launched and not self._pending:
                    self._lock.wait(timeout=0.0002 if self._in_flight else 0.01)

    def _poll(self):
        done = [b for b in self._in_flight if b.event.query()]
        for batch in done:
            self._in_flight.remove(batch)
            self._in_flight_bytes -= batch.nbytes
            now = time.perf_counter()
            code = int(batch.host["error"].numpy()[0])
            for index, job in enumerate(batch.jobs):
                if code:
                    job.future.set_exception(ValueError(f"invalid request in batch (error bits {code:#x})"))
                    continue
                values = self._unpack(batch, index)
                job.future.set_result(Response(batch.kind, values, 1000 * (now - job.arrival), len(batch.jobs)))

    def _admit(self):
        """Pop admitted jobs (FIFO) grouped by kind."""
        groups = {"panoptic": [], "prefix": []}
        with self._lock:
            while self._pending and len(self._in_flight) < len(self._streams):
                job = self._pending[0]
                need = self.footprint(job.request)
                if need > self.memory_budget:
                    self._pending.popleft()
                    job.future.set_exception(ValueError(
                        f"request needs {need} bytes of device memory, above the {self.memory_budget}-byte budget"))
                    continue
                admitted = sum(self.footprint(j.request) for g in groups.values() for j in g)
                if self._in_flight_bytes + admitted + need > self.memory_budget:
                    break
                group = groups[job.request.kind]
                if len(group) >= self.max_batch:
                    break
                group.append(self._pending.popleft())
        return groups

    def _launch(self):
        groups = self._admit()
        launched = False
        for kind, jobs in groups.items():
            if not jobs:
                continue
            free = [s for s in self._streams if all(b.stream is not s for b in self._in_flight)]
            stream = free[0] if free else self._streams[self.batches % len(self._streams)]
            try:
                batch = (self._launch_panoptic if kind == "panoptic" else self._launch_prefix)(jobs, stream)
            except Exception as error:  # report on every request of the batch
                for job in jobs:
                    job.future.set_exception(error)
                continue
            self._in_flight.append(batch)
            self._in_flight_bytes += batch.nbytes
            self.peak_in_flight_bytes = max(self.peak_in_flight_bytes, self._in_flight_bytes)
            self.batches += 1
            launched = True
        return launched

    def _upload(self, blobs, stream):
        """Copy request blobs into one device arena; returns (arena, byte offsets)."""
        offsets, total = [], 0
        for blob in blobs:
            offsets.append(total)
            total += _round(blob.numel())
        arena = torch.empty(max(total, 1), dtype=torch.uint8, device=self.device)
        for blob, off in zip(blobs, offsets):
            arena[off: off + blob.numel()].copy_(blob, non_blocking=True)
        return arena, offsets

    def _meta(self, parts):
        """Pack small int32/uint8 numpy arrays into one pinned upload; returns device views in order."""
        sizes = [_round(p.nbytes, 16) for p in parts]
        host = _pinned(sum(sizes))
        view = host.numpy()
        off = 0
        for p, size in zip(parts, sizes):
            view[off: off + p.nbytes] = p.reshape(-1).view(np.uint8)
            off += size
        dev = host.to(self.device, non_blocking=True)
        out, off = [], 0
        for p, size in zip(parts, sizes):
            dtype = {np.dtype(np.int32): torch.int32, np.dtype(np.uint8): torch.uint8,
                     np.dtype(np.int64): torch.int64, np.dtype(np.float64): torch.float64}[p.dtype]
            out.append(dev[off: off + p.nbytes].view(dtype))
            off += size
        return out, host

    def _launch_panoptic(self, jobs, stream):
        reqs = [j.request for j in jobs]
        B, C = len(reqs), self.num_classes
        with torch.cuda.stream(stream):
            arena, offsets = self._upload([r.blob for r in reqs], stream)
            Gs = np.array([len(r.target_classes) for r in reqs], np.int64)
            Ps = np.array([len(r.pred_classes) for r in reqs], np.int64)
            hw = np.array([r.hw for r in reqs], np.int64)
            d = np.zeros((B, SEG_FIELDS), np.int64)
            base = arena.data_ptr() + np.array(offsets, np.int64)
            d[:, TARGET] = base
            d[:, PRED] = base + np.array([r.span for r in reqs], np.int64)
            d[:, PIXELS] = hw
            d[:, MASK_STRIDE] = 16
            chunks = -(-hw // SEG_CHUNK)
            d[:, CHUNK_BEGIN] = np.cumsum(chunks) - chunks
            d[:, SLOT_BEGIN] = np.cumsum(Gs) - Gs
            d[:, PSLOT_BEGIN] = np.cumsum(Ps) - Ps
            pan = Gs * Ps
            d[:, PAIR_BEGIN] = np.cumsum(pan) - pan
            d[:, G] = Gs
            d[:, P] = Ps
            d[:, FLAGS] = 3
            (descs, gc, pc, crowd), host_meta = self._meta([
                d, np.concatenate([r.target_classes for r in reqs]), np.concatenate([r.pred_classes for r in reqs]),
                np.concatenate([r.crowd for r in reqs])])
            ints, longs = dict(dtype=torch.int32, device=self.device), dict(dtype=torch.int64, device=self.device)
            pairs = torch.empty(max(int(pan.sum()), 1), **ints)
            areas = torch.empty(int((Gs + Ps).sum()), **longs)
            matched = torch.empty(int(Gs.sum()), **ints)
            stats = torch.zeros((3, B, C), **longs)
            sums = torch.zeros((B, C), dtype=torch.float64, device=self.device)
            pq = torch.empty(B, dtype=torch.float64, device=self.device)
            error = torch.zeros(1, **ints)
            h = N.stream_handle(self.device)
            N.call("pe_seg_pass", N.ptr(descs), B, int(chunks.sum()), None, N.ptr(pairs), int(pan.sum()), None, 0,
                   int(pan.max()), 0, 1, N.ptr(error), h)
            N.call("pe_seg_score", N.ptr(descs), B, int(Ps.max()), N.ptr(pairs), None, N.ptr(gc), N.ptr(pc),
                   N.ptr(crowd), N.ptr(areas), N.ptr(matched), N.ptr(stats[0]), N.ptr(stats[1]), N.ptr(stats[2]),
                   N.ptr(sums), None, C, N.ptr(self._things_u8), None, None, None, None, None, None, None,
                   int(self.validate), 1, N.ptr(error), h)
            t = self.totals
            N.call("pe_reward_pq", N.ptr(stats[0]), N.ptr(stats[1]), N.ptr(stats[2]), N.ptr(sums), B, C, N.ptr(pq),
                   N.ptr(t["tp"]), N.ptr(t["fp"]), N.ptr(t["fn"]), N.ptr(t["iou_sum"]), h)
            host_pq = torch.empty(B, dtype=torch.float64, pin_memory=True)
            host_pq.copy_(pq, non_blocking=True)
            host_err = torch.empty(1, dtype=torch.int32, pin_memory=True)
            host_err.copy_(error, non_blocking=True)
            event = torch.cuda.Event()
            event.record(stream)
        batch = _Batch("panoptic", jobs, stream, event, sum(self.footprint(r) for r in reqs))
        batch.keep = [arena, descs, gc, pc, crowd, host_meta, pairs, areas, matched, stats, sums, pq, error]
        batch.host = dict(pq=host_pq, error=host_err)
        return batch

    def _launch_prefix(self, jobs, stream):
        reqs = [j.request for j in jobs]
        B, C, T = len(reqs), self.num_classes, len(self.thresholds)
        with torch.cuda.stream(stream):
            arena, offsets = self._upload([r.blob for r in reqs], stream)
            n = np.array([r.n for r in reqs], np.int64)
            Gs = np.array([len(r.target_classes) for r in reqs], np.int64)
            q = np.array([len(r.points) for r in reqs], np.int64)
            hw = np.array([r.hw for r in reqs], np.int64)
            base = arena.data_ptr() + np.array(offsets, np.int64)
            d = np.zeros((B, PF.FIELDS), np.int64)
            d[:, PF.TARGET] = base
            d[:, PF.MASKS] = base + np.array([r.span for r in reqs], np.int64)
            d[:, PF.PIXELS] = hw
            d[:, PF.STRIDE] = [r.pitch for r in reqs]
            chunks = -(-hw // PF.CHUNK)
            d[:, PF.CHUNK_BEGIN] = np.cumsum(chunks) - chunks
            d[:, PF.NMASK] = n
            d[:, PF.NSLOT] = Gs
            d[:, PF.DET_BEGIN] = np.cumsum(n) - n
            d[:, PF.SLOT_BEGIN] = np.cumsum(Gs) - Gs
            d[:, PF.Q_BEGIN] = np.cumsum(q) - q
            d[:, PF.NQ] = q
            cells = q * Gs * (n + 1)
            d[:, PF.PAIR_BEGIN] = np.cumsum(cells) - cells
            d[:, PF.RAW_BEGIN] = np.cumsum(n * Gs) - n * Gs
            d[:, PF.FLAGS] = 3
            d[:, PF.STEP_BEGIN] = np.cumsum(n + 1) - (n + 1)
            d[:, PF.COUNT_BEGIN] = np.arange(B) * T * C * 2
            steps = np.full(int((n + 1).sum()), -1, np.int32)
            for b, r in enumerate(reqs):
                for index, k in enumerate(r.points):
                    steps[int(d[b, PF.STEP_BEGIN]) + k] = index
            (descs, step_q, classes, gc, crowd), host_meta = self._meta([
                d, steps, np.concatenate([r.classes for r in reqs]) if n.sum() else np.zeros(1, np.int32),
                np.concatenate([r.target_classes for r in reqs]), np.concatenate([r.crowd for r in reqs])])
            R = int(q.sum())
            ints, longs = dict(dtype=torch.int32, device=self.device), dict(dtype=torch.int64, device=self.device)
            doubles = dict(dtype=torch.float64, device=self.device)
            out = dict(tp=torch.empty((R, C), **longs), fp=torch.empty((R, C), **longs),
                       fn=torch.empty((R, C), **longs), sums=torch.empty((R, C), **doubles),
                       confusion=torch.empty((R, C, C + 1), **longs), itp=torch.empty((R, T, C), **longs),
                       ifp=torch.empty((R, T, C), **longs), ifn=torch.empty((R, T, C), **longs),
                       precision=torch.empty((R, T, C), **doubles), recall=torch.empty((R, T, C), **doubles),
                       values=torch.empty((R, 4, C), **doubles), summaries=torch.empty((R, 3, 3), **doubles),
                       counts=torch.empty((R, 3), **longs), miou=torch.empty((R,), **doubles))
            ga = torch.empty(int(Gs.sum()), **ints)
            raw = torch.empty(max(int((n * Gs).sum()), 1), **ints)
            pairs = torch.empty(max(int(cells.sum()), 1), **ints)
            counters = torch.empty(B * T * C * 2, **ints)
            error = torch.zeros(1, **ints)
            N.call("pe_prefix", N.ptr(descs), B, int(chunks.sum()), R, int(Gs.max()), int(n.max()) + 1,
                   int((Gs * (n + 1)).max()), N.ptr(step_q), N.ptr(classes), N.ptr(gc), N.ptr(crowd),
                   N.ptr(self._things_u8), N.ptr(self._thr), T, C, N.ptr(ga), ga.numel(), N.ptr(raw),
                   int((n * Gs).sum()), N.ptr(pairs), int(cells.sum()), N.ptr(counters), counters.numel(),
                   N.ptr(out["tp"]), N.ptr(out["fp"]), N.ptr(out["fn"]), N.ptr(out["sums"]), N.ptr(out["confusion"]),
                   N.ptr(out["itp"]), N.ptr(out["ifp"]), N.ptr(out["ifn"]), N.ptr(out["precision"]),
                   N.ptr(out["recall"]), N.ptr(out["values"]), N.ptr(out["summaries"]), N.ptr(out["counts"]),
                   N.ptr(out["miou"]), int(self.validate), N.ptr(error), N.stream_handle(self.device))
            host = {}
            for key in _PREFIX_KEYS + (_PREFIX_FULL_KEYS if self.full_results else ()):
                host[key] = torch.empty(out[key].shape, dtype=out[key].dtype, pin_memory=True)
                host[key].copy_(out[key], non_blocking=True)
            host["error"] = torch.empty(1, dtype=torch.int32, pin_memory=True)
            host["error"].copy_(error, non_blocking=True)
            event = torch.cuda.Event()
            event.record(stream)
        batch = _Batch("prefix", jobs, stream, event, sum(self.footprint(r) for r in reqs))
        batch.keep = [arena, descs, step_q, classes, gc, crowd, host_meta, out, ga, raw, pairs, counters, error]
        batch.host = host
        batch.layout = d[:, PF.Q_BEGIN].copy()
        return batch

    def _unpack(self, batch, index):
        if batch.kind == "panoptic":
            return dict(pq=float(batch.host["pq"].numpy()[index]))
        req = batch.jobs[index].request
        first = int(batch.layout[index])
        host = {key: value.numpy() for key, value in batch.host.items()}
        snapshots = []
        for offset, k in enumerate(req.points):
            r = first + offset
            s, n = host["summaries"][r], host["counts"][r]
            snap = {name: dict(pq=float(s[i, 0]), sq=float(s[i, 1]), rq=float(s[i, 2]), n=int(n[i]))
                    for i, name in enumerate(("All", "Things", "Stuff"))}
            snap.update(prefix=k, miou=float(host["miou"][r]),
                        instance=dict(iou_thresholds=np.array(self.thresholds), tp=host["itp"][r].copy(),
                                      fp=host["ifp"][r].copy(), fn=host["ifn"][r].copy(),
                                      precision=host["precision"][r].copy(), recall=host["recall"][r].copy()))
            if self.full_results:
                v = host["values"][r]
                snap.update(tp=host["tp"][r].copy(), fp=host["fp"][r].copy(), fn=host["fn"][r].copy(),
                            iou_sum=host["sums"][r].copy(), confusion=host["confusion"][r].copy(),
                            per_class={name: v[i].copy() for i, name in enumerate(("pq", "sq", "rq", "iou"))})
            snapshots.append(snap)
        return dict(snapshots=snapshots)


def serve(server: RewardServer, requests, arrivals):
    """Submit `requests` at `arrivals` (seconds from now, ascending) and wait for all.

    Returns (responses, summary) where summary has throughput and p50/p99 latency.
    """
    server.start()
    t0 = time.perf_counter()
    futures = []
    for request, at in zip(requests, arrivals):
        target = t0 + at
        while True:
            now = time.perf_counter()
            if now >= target:
                break
            if target - now > 0.0005:
                time.sleep(target - now - 0.0003)
        futures.append(server.submit(request, arrival=target))
    responses = [f.result() for f in futures]
    wall = time.perf_counter() - t0
    lat = sorted(r.latency_ms for r in responses)
    pick = lambda p: lat[min(len(lat) - 1, int(round(p * (len(lat) - 1))))]  # noqa: E731
    summary = dict(requests=len(responses), wall_s=wall, throughput=len(responses) / wall,
                   p50_ms=pick(0.50), p99_ms=pick(0.99), mean_ms=statistics.fmean(lat),
                   batches=server.batches, peak_in_flight_bytes=server.peak_in_flight_bytes,
                   mean_batch=statistics.fmean(r.batch_size for r in responses))
    return responses, summary
