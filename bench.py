#!/usr/bin/env python
"""Benchmark: combined PQ + mIoU + mask AP images/s on GB300 (batched graph path vs plain per-image path).

Workload: SegmentationEvaluator over 256 uneven images (sides 320-1024, target
slots 10-150, detections 5-100, 133 classes; seeded synthetic data with
COCO-like shapes). One step = reset + update + compute over the whole batch.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Prints one JSON line (rank 0). `value` replays a CUDA graph of the step with
inputs resident in HBM; `e2e` adds the host->device upload of the batch arena
from pinned memory and the device->host read of the headline metrics every
step. `--impl reference` times the reference algorithm's CPU implementation
(the numpy oracle, all host cores) on bounded samples of the same workload.
"""

from __future__ import annotations

import argparse
import json
import math
import multiprocessing as mp
import os
import shutil
import statistics
import subprocess
import sys
import time
from collections.abc import Mapping, Sequence
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "images/s combined PQ+mIoU+AP, batched vs plain on 1 GB300; reward p50/p99 ms"
NUM_CLASSES, THINGS = 133, 80
WORKLOAD = ("SegmentationEvaluator (combined PQ+mIoU+mask AP) over 256 uneven images, sides U[320,1024], "
            "target slots 10-150, detections 5-100, 133 classes (80 things)")


def parse():
    p = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=400)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=("gb300", "reference"), default="gb300")
    p.add_argument("--images", type=int, default=256)
    p.add_argument("--seed", type=int, default=4)
    p.add_argument("--plain-steps", type=int, default=2)
    p.add_argument("--cpu-sample", type=int, default=256, help="images timed on the CPU oracle (baseline leg)")
    p.add_argument("--serve-requests", type=int, default=4000, help="requests of the reward serving run (0: skip)")
    p.add_argument("--serve-rate", type=float, default=2000.0, help="mean Poisson arrival rate, requests/s")
    p.add_argument("--instance-images", type=int, default=32, help="images of the mask AP batch (0: skip)")
    p.add_argument("--prefix-images", type=int, default=16, help="images of the generation-prefix batch (0: skip)")
    p.add_argument("--published", type=int, default=1,
                   help="1: time the shapes of the reference's recorded A100 combined timings (0: skip)")
    p.add_argument("--panoptic-batches", type=int, default=8,
                   help="16-image COCO-shape batches of the PanopticEvaluator section (0: skip)")
    p.add_argument("--reference-cuda", type=int, default=1,
                   help="1: time the reference's own CUDA extension on the same workloads (baseline/_ref)")
    p.add_argument("--reference-cuda-timeout", type=float, default=900.0)
    p.add_argument("--reference-cpu", type=int, default=1,
                   help="1: time the reference's own CPU evaluators (torch) on bounded samples (baseline/_ref)")
    p.add_argument("--case", choices=("combined", "instance", "panoptic", "prefix"), default=None,
                   help="profiling mode: run --case-steps steps of one workload on --case-images images, no JSON")
    p.add_argument("--case-images", type=int, default=32)
    p.add_argument("--case-steps", type=int, default=3)
    return p.parse_args()


def rank_info():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


PARITY_TOL = 1e-12  # FP64 metrics against the oracle; every integer quantity is compared exactly


class Parity:
    """Result-against-oracle comparison of one bench section.

    Walks the oracle's result tree (dicts, lists, arrays, scalars): integer and
    bool leaves must be equal, floating-point leaves within ``PARITY_TOL``
    absolute, NaN only where the oracle has NaN. Keys the oracle lacks are not
    compared.
    """

    def __init__(self):
        self.int_exact = True
        self.max_abs = 0.0
        self.leaves = 0
        self.failures = []

    def _fail(self, message):
        self.int_exact = self.int_exact and not message.startswith("int")
        if len(self.failures) < 5:
            self.failures.append(message)

    def compare(self, actual, expected, path="result"):
        if isinstance(expected, Mapping):
            for key in expected:
                if key not in actual:
                    self._fail(f"missing {path}/{key}")
                else:
                    self.compare(actual[key], expected[key], f"{path}/{key}")
            return self
        if isinstance(expected, Sequence) and not isinstance(expected, str):
            if len(actual) != len(expected):
                self._fail(f"length {path}: {len(actual)} != {len(expected)}")
                return self
            for i, (a, e) in enumerate(zip(actual, expected)):
                self.compare(a, e, f"{path}/{i}")
            return self
        a = actual.detach().cpu().numpy() if hasattr(actual, "detach") else np.asarray(actual)
        e = np.asarray(expected)
        self.leaves += 1
        if a.shape != e.shape:
            self._fail(f"shape {path}: {a.shape} != {e.shape}")
            return self
        if e.dtype.kind in "iub":
            if not np.array_equal(a.astype(np.int64), e.astype(np.int64)):
                self._fail(f"int {path}")
            return self
        a, e = a.astype(np.float64), e.astype(np.float64)
        if not np.array_equal(np.isnan(a), np.isnan(e)):
            self._fail(f"nan {path}")
            self.max_abs = math.inf
            return self
        finite = ~np.isnan(e)
        if finite.any():
            diff = float(np.max(np.abs(a[finite] - e[finite])))
            self.max_abs = max(self.max_abs, diff)
            if not diff <= PARITY_TOL:
                self._fail(f"fp64 {path}: {diff:.3e}")
        return self

    def ok(self):
        return not self.failures

    def summary(self, against):
        return {"checked": True, "against": against, "int_exact": self.int_exact, "max_abs_fp64": self.max_abs,
                "tolerance_fp64": PARITY_TOL, "leaves": self.leaves, "ok": self.ok()}

    def require(self, section):
        if not self.ok():
            raise RuntimeError(f"{section}: result differs from the oracle: {self.failures}")


def generate(args, rank, pool):
    from panoptic_evaluator_gb300 import synthetic
    return synthetic.segmentation_batch(seed=args.seed + 1000 * rank, images=args.images, pool=pool)


SERVE_PANOPTIC, SERVE_PREFIX = 256, 32  # distinct requests, replayed in a seeded random order
SERVE_POINTS = list(range(8, 65, 8))


def generate_serving(args, pool):
    """Distinct reward requests: COCO-shape panoptic images and 64-mask generation prefixes, sides U[256,1024]."""
    from functools import partial

    from panoptic_evaluator_gb300 import synthetic
    pan = pool.map(partial(synthetic.segmentation_one, args.seed + 77, side=(256, 1024), slots=(10, 100),
                           dets=(0, 0)), range(SERVE_PANOPTIC), chunksize=8)
    pre = pool.map(partial(synthetic.prefix_one, args.seed + 78, side=(256, 1024), masks=64, slots=101),
                   range(SERVE_PREFIX), chunksize=1)
    return pan, pre


def _serving_pq_oracle(im):
    """Oracle per-image PQ of one panoptic_quality request (evaluator.py:471-544)."""
    from oracle import panoptic as opan
    return float(opan.panoptic_quality(im.pred[None], im.pred_classes[None], im.target[None],
                                       im.target_classes[None], im.crowd[None], NUM_CLASSES,
                                       validate_inputs=False)[0])


def _prefix_oracle(im):
    """Oracle snapshots of one generation-prefix image at checkpoints 8, 16, ..., 64 (prefix.py:63-120)."""
    from oracle import prefix as opre
    return opre.image_prefixes(im.target, im.target_classes, im.crowd, im.masks, im.classes,
                               np.array(isthing(), bool), NUM_CLASSES, np.array([0.5, 0.75]), set(SERVE_POINTS))


def serving_oracles(pan, pre, pool):
    return pool.map(_serving_pq_oracle, pan, chunksize=8), pool.map(_prefix_oracle, pre, chunksize=1)


def run_serving(args, pan, pre, dev, oracles):
    """Open-loop Poisson run of the reward server; every distinct request checked against the oracle."""
    import torch

    import panoptic_evaluator_gb300 as pe
    from panoptic_evaluator_gb300.serving import PanopticRequest, PrefixRequest, RewardServer, serve
    requests = [PanopticRequest(im.pred, im.pred_classes, im.target, im.target_classes, im.crowd) for im in pan]
    requests += [PrefixRequest(im.masks, im.classes, im.target, im.target_classes, im.crowd,
                               checkpoints=SERVE_POINTS) for im in pre]
    rng = np.random.default_rng(args.seed + 79)
    # Half of the arrivals are panoptic_quality requests, half prefix requests.
    kinds = rng.random(args.serve_requests) < 0.5
    picks = [int(rng.integers(0, SERVE_PANOPTIC)) if k else SERVE_PANOPTIC + int(rng.integers(0, SERVE_PREFIX))
             for k in kinds]
    arrivals = np.cumsum(rng.exponential(1.0 / args.serve_rate, args.serve_requests))
    server = RewardServer(NUM_CLASSES, isthing=isthing(), device=dev, memory_budget=8 << 30, max_batch=64, trace=True)
    with server:
        warm = min(200, args.serve_requests)
        serve(server, [requests[i] for i in picks[:warm]], arrivals[:warm] - arrivals[0])
        server.batches = 0
        server.peak_in_flight_bytes = 0
        server.trace.clear()
        responses, summary = serve(server, [requests[i] for i in picks], arrivals)
        trace_rows = list(server.trace)
        # The same arrivals once more with the objects that exist before the run frozen out of the cyclic
        # collector's scans (gc.freeze: collections still run over what the run allocates).
        frozen = serve(server, [requests[i] for i in picks], arrivals, freeze_gc=True)[1]
        server.trace[:] = trace_rows
    trace = {}
    for kind in ("panoptic", "prefix"):
        rows = [t for t in server.trace if t["kind"] == kind]
        if rows:
            trace[kind] = {key: {"p50": float(np.percentile([t[key] for t in rows], 50)),
                                 "p99": float(np.percentile([t[key] for t in rows], 99))}
                           for key in ("size", "queue_ms", "launch_ms", "device_ms", "detect_ms")}
    # Every response against the oracle's result for its request: PQ of panoptic_quality requests, and
    # every checkpoint snapshot (PQ/SQ/RQ groups, mIoU, instance counts, precision, recall) of prefixes.
    pq_oracle, prefix_oracle = oracles
    parity = Parity()
    for response, index in zip(responses, picks):
        if index < SERVE_PANOPTIC:
            parity.compare(response.values["pq"], pq_oracle[index], f"panoptic[{index}]/pq")
        else:
            expected = prefix_oracle[index - SERVE_PANOPTIC]
            parity.compare(response.values["snapshots"], [
                {key: snap[key] for key in ("All", "Things", "Stuff", "prefix", "miou", "instance")}
                for snap in expected], f"prefix[{index - SERVE_PANOPTIC}]")
    parity.require("serving")
    # Plain path: panoptic_quality on each distinct panoptic image, one call per image.
    worst = 0.0
    for index in sorted(set(i for i in picks if i < SERVE_PANOPTIC)):
        im = pan[index]
        plain = pe.panoptic_quality(
            pe.PanopticBatch(torch.from_numpy(im.pred[None]).to(dev), torch.from_numpy(im.pred_classes[None]).to(dev)),
            pe.PanopticBatch(torch.from_numpy(im.target[None]).to(dev),
                             torch.from_numpy(im.target_classes[None]).to(dev), torch.from_numpy(im.crowd[None]).to(dev)),
            NUM_CLASSES)
        got = [r.values["pq"] for r, i in zip(responses, picks) if i == index]
        worst = max(worst, max(abs(g - float(plain[0])) for g in got))
    return {
        "parity": parity.summary(f"oracle, all {len(responses)} responses ({len(set(picks))} distinct requests)"),
        "offered_rate": args.serve_rate, "requests": summary["requests"], "throughput": summary["throughput"],
        "unit": "requests/s", "p50_ms": summary["p50_ms"], "p99_ms": summary["p99_ms"], "mean_ms": summary["mean_ms"],
        "max_ms": summary["max_ms"], "gc_paused": summary["gc_paused"], "gc_frozen": summary["gc_frozen"],
        "with_gc_freeze": {"p50_ms": frozen["p50_ms"], "p99_ms": frozen["p99_ms"], "max_ms": frozen["max_ms"],
                           "throughput": frozen["throughput"],
                           "note": "same run with the objects alive before it frozen out of the collector's scans "
                                   "(serve(freeze_gc=True)); the collector stays on"},
        "batches": summary["batches"], "mean_batch": summary["mean_batch"],
        "peak_in_flight_bytes": summary["peak_in_flight_bytes"],
        "mix": "50% per-image panoptic_quality (COCO shape, sides U[256,1024], slots 10-100, 133 classes), 50% "
               "generation prefixes (64 masks, checkpoints 8..64 step 8)",
        "distinct_requests": {"panoptic": SERVE_PANOPTIC, "prefix": SERVE_PREFIX},
        "max_abs_pq_diff_vs_plain": worst,
        "batch_trace": trace,
    }


def generate_instance(args, pool):
    """COCO-like mask AP batch: sides U[480,640], 80 classes, 1-50 targets and 100 predictions per image."""
    from functools import partial

    from panoptic_evaluator_gb300 import synthetic
    return pool.map(partial(synthetic.instance_one, args.seed + 90), range(args.instance_images), chunksize=1)


def _instance_oracle(im):
    """One image through the oracle's InstanceEvaluator (instance.py:78-203 CPU branch)."""
    from oracle import instance as oinst
    oracle = oinst.InstanceOracle(80, validate=False)
    return oracle.update([im.pred_masks], [im.pred_classes], [im.scores], [im.gt_masks], [im.gt_classes],
                         [im.crowd])


def instance_oracle(images, pool):
    """The oracle's AP/AR over the batch, images evaluated in parallel and merged in order."""
    from oracle import instance as oinst
    total = oinst.InstanceOracle(80, validate=False)
    for part in pool.map(_instance_oracle, images, chunksize=1):
        total.records.extend(part.records)
        total.counts += part.counts
    return total.compute()


def run_instance(args, images, dev, peak, oracle, ours):
    """InstanceEvaluator update + compute over the batch (device-resident masks) vs one update per image."""
    import torch

    import panoptic_evaluator_gb300 as pe
    from panoptic_evaluator_gb300 import _native

    def batch(items):
        return (pe.InstanceBatch([torch.from_numpy(i.pred_masks).to(dev) for i in items],
                                 [torch.from_numpy(i.pred_classes).to(dev) for i in items],
                                 [torch.from_numpy(i.scores).to(dev) for i in items]),
                pe.InstanceBatch([torch.from_numpy(i.gt_masks).to(dev) for i in items],
                                 [torch.from_numpy(i.gt_classes).to(dev) for i in items],
                                 crowd=[torch.from_numpy(i.crowd).to(dev) for i in items]))

    pred, target = batch(images)
    ev = pe.InstanceEvaluator(80, device=dev, validate=False)
    from panoptic_evaluator_gb300 import tuning
    contract_tuning = tuning.tune_contract(ev, pred, target, repeats=3)

    def step():
        ev.reset()
        ev.update(pred, target)
        return ev.compute()["ap"]

    events = []
    original = _native.call

    def timed_call(name, *a):
        if name != "pe_inst_contract":
            return original(name, *a)
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        out = original(name, *a)
        e.record()
        events.append((s, e))
        return out

    for _ in range(args.warmup):
        step()
    _native.call = timed_call
    try:
        for _ in range(5):
            step()
    finally:
        _native.call = original
    torch.cuda.synchronize()
    before = _native.launch_count()
    step()
    torch.cuda.synchronize()
    launches = _native.launch_count() - before
    steps = max(5, args.steps // 10)
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    start.record()
    for _ in range(steps):
        ap = step()
    end.record()
    end.synchronize()
    ms = start.elapsed_time(end) / steps
    singles = [batch([i]) for i in images]
    plain = pe.InstanceEvaluator(80, device=dev, validate=False)

    def plain_step():
        plain.reset()
        for p, t in singles:
            plain.update(p, t)
        return plain.compute()["ap"]

    plain_step()
    torch.cuda.synchronize()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record()
    plain_ap = plain_step()
    e.record()
    e.synchronize()
    ms_plain = s.elapsed_time(e)
    torch.testing.assert_close(plain_ap, ap, rtol=1e-12, atol=1e-12)
    full = ev.compute()
    parity = Parity().compare(full, oracle)
    parity.require("instance")
    ours["instance"] = (len(images) / (ms / 1e3), full)
    algo = sum((i.pred_masks.shape[0] + i.gt_masks.shape[0]) * i.pred_masks.shape[1] * i.pred_masks.shape[2]
               for i in images)
    kernel_ms = statistics.median(a.elapsed_time(b) for a, b in events)
    achieved = algo / (kernel_ms / 1e3) / 1e9
    return {
        "workload": f"InstanceEvaluator (COCO mask AP) over {len(images)} images, sides U[480,640], 80 classes, "
                    "1-50 targets (2% crowd) and 100 predictions per image",
        "value": len(images) / (ms / 1e3), "unit": "images/s", "ms_per_step": ms,
        "step": "reset + update (sort, tensor-core contraction, prep, matching) + compute, masks resident in HBM",
        "plain": {"value": len(images) / (ms_plain / 1e3), "unit": "images/s", "ms_per_step": ms_plain,
                  "mode": "one update() per image"},
        "gpu_launches_per_step": launches,
        "ap": float(ap),
        "parity": parity.summary(f"oracle InstanceEvaluator over all {len(images)} images"),
        "roofline": {"bound": "hbm", "kernel": "inst_contract_kernel (tcgen05 kind::f8f6f4)", "achieved": achieved,
                     "peak": peak, "unit": "GB/s", "frac": achieved / peak, "kernel_ms": kernel_ms,
                     "algorithmic_bytes_per_launch": algo},
        "contract_tuning": {"choice": {"tma_bucket": contract_tuning["tma_bucket"],
                                       "tma_cost": contract_tuning["tma_cost"]},
                            "candidates_contract_ms": contract_tuning["candidates"],
                            "note": "pe_inst_contract timed per CTA-split weight of TMA-loaded blocks on this batch "
                                    "(tuning.tune_contract); the fastest is used for the timings above"},
    }


def generate_prefix(args, pool):
    """Same-size generation-prefix batch: 64 masks per image, side drawn once in [256, 1024], 101 target slots."""
    from panoptic_evaluator_gb300 import synthetic
    return synthetic.prefix_batch(seed=args.seed + 300, images=args.prefix_images, masks=64, pool=pool)


def run_prefix(args, images, dev, peak, oracle, ours):
    """segmentation_prefixes over the batch, checkpoints 8, 16, ..., 64; device-resident inputs."""
    import torch

    import panoptic_evaluator_gb300 as pe
    from panoptic_evaluator_gb300 import _native
    target = pe.PanopticBatch(torch.from_numpy(np.stack([i.target for i in images])).to(dev),
                              torch.from_numpy(np.stack([i.target_classes for i in images])).to(dev),
                              torch.from_numpy(np.stack([i.crowd for i in images])).to(dev))
    pred = pe.InstanceBatch([torch.from_numpy(i.masks).to(dev) for i in images],
                            [torch.from_numpy(i.classes).to(dev) for i in images])
    points = list(range(8, 65, 8))

    def step():
        return pe.segmentation_prefixes(pred, target, NUM_CLASSES, isthing=isthing(), checkpoints=points,
                                        validate=False)

    for _ in range(args.warmup):
        step()
    events, original = [], _native.call

    def timed_call(name, *a):
        if name != "pe_prefix":
            return original(name, *a)
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        out = original(name, *a)
        e.record()
        events.append((s, e))
        return out

    _native.call = timed_call
    try:
        for _ in range(3):
            step()
    finally:
        _native.call = original
    torch.cuda.synchronize()
    steps = max(5, args.steps // 20)
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    start.record()
    for _ in range(steps):
        result = step()
    end.record()
    end.synchronize()
    ms = start.elapsed_time(end) / steps
    parity = Parity().compare(result, oracle)
    parity.require("prefix")
    ours["prefix"] = (len(images) / (ms / 1e3), result)
    hw = images[0].target.size
    algo = sum((4 + len(i.masks)) * hw for i in images)
    call_ms = statistics.median(a.elapsed_time(b) for a, b in events)
    achieved = algo / (call_ms / 1e3) / 1e9
    return {
        "workload": f"segmentation_prefixes over {len(images)} images of {images[0].target.shape[0]} x "
                    f"{images[0].target.shape[1]}, 64 generation-ordered masks each, checkpoints 8..64 step 8, "
                    "133 classes",
        "value": len(images) / (ms / 1e3), "unit": "images/s", "ms_per_step": ms,
        "pq_last": float(result[0][-1]["All"]["pq"]), "gc_paused": False,
        "parity": parity.summary(f"oracle snapshots of all {len(images)} images at every checkpoint"),
        "pe_prefix": {"ms": call_ms, "algorithmic_bytes": algo, "effective_gbs": achieved, "frac": achieved / peak,
                      "note": "one pe_prefix call (owner pass, scan, checkpoint scoring, matching, summaries); "
                              "bytes = (4 + N) x H x W per image"},
    }


# The reference's recorded combined timings (A100 80GB PCIe, DEVELOPMENT.md:39-45): 8 images, 15
# categories, validation off, median over seven rounds of reset + update + compute.
PUBLISHED = ((256, 384, 64, 64, 3.776), (512, 768, 256, 256, 5.350))
# Its recorded segmentation_prefixes timings (A100, benchmarks/prefix_results.md:46-70): one image,
# validation off, seven rounds; ms per sequence with every prefix and with every 8th (and the last).
PUBLISHED_PREFIX = ((128, 192, 16, 1.39, 0.54), (256, 384, 64, 4.30, 1.50), (512, 768, 64, 4.32, 1.59))


def run_published(args, dev):
    """SegmentationEvaluator on the shapes of the reference's recorded A100 timings, timed the same way."""
    import torch

    import panoptic_evaluator_gb300 as pe
    from panoptic_evaluator_gb300 import synthetic
    rows = []
    for h, w, segments, dets, a100_ms in PUBLISHED:
        images, things = synthetic.grid_batch(seed=args.seed + 400, images=8, height=h, width=w, segments=segments,
                                              detections=dets, num_classes=15)
        t = lambda key: torch.from_numpy(np.stack([getattr(i, key) for i in images])).to(dev)  # noqa: E731
        target = pe.PanopticBatch(t("target"), t("target_classes"), t("crowd"))
        prediction = pe.PanopticBatch(t("pred"), t("pred_classes"))
        detections = pe.InstanceBatch([torch.from_numpy(i.det_masks).to(dev) for i in images],
                                      [torch.from_numpy(i.det_classes).to(dev) for i in images],
                                      [torch.from_numpy(i.scores).to(dev) for i in images])
        ev = pe.SegmentationEvaluator(15, isthing=things, device=dev, validate=False)

        def step():
            ev.reset()
            ev.update(prediction, detections, target)
            return ev.compute()

        for _ in range(3):
            step()
        times = []
        for _ in range(7):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            result = step()
            torch.cuda.synchronize()
            times.append((time.perf_counter() - t0) * 1e3)
        ms = statistics.median(times)
        rows.append({"images": 8, "height": h, "width": w, "segments": segments, "detections": dets,
                     "ms_per_batch": ms, "reference_a100_ms": a100_ms, "a100_over_gb300": a100_ms / ms,
                     "pq": float(result["All"]["pq"]), "ap": float(result["instance"]["ap"])})
    prefix_rows = []
    for h, w, n, every_ms, eighth_ms in PUBLISHED_PREFIX:
        im = synthetic.prefix_one(args.seed + 500, 0, masks=n, fixed_hw=(h, w))
        target = pe.PanopticBatch(torch.from_numpy(im.target[None]).to(dev),
                                  torch.from_numpy(im.target_classes[None]).to(dev),
                                  torch.from_numpy(im.crowd[None]).to(dev))
        pred = pe.InstanceBatch([torch.from_numpy(im.masks).to(dev)], [torch.from_numpy(im.classes).to(dev)])
        for label, points, a100_ms in (("every prefix", list(range(1, n + 1)), every_ms),
                                       ("every 8th prefix", sorted(set(range(8, n + 1, 8)) | {n}), eighth_ms)):
            def run():
                return pe.segmentation_prefixes(pred, target, NUM_CLASSES, isthing=isthing(), checkpoints=points,
                                                validate=False)
            for _ in range(3):
                run()
            times = []
            for _ in range(7):
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                out = run()
                torch.cuda.synchronize()
                times.append((time.perf_counter() - t0) * 1e3)
            ms = statistics.median(times)
            prefix_rows.append({"height": h, "width": w, "masks": n, "checkpoints": label, "ms_per_sequence": ms,
                                "reference_a100_ms": a100_ms, "a100_over_gb300": a100_ms / ms,
                                "pq_last": float(out[0][-1]["All"]["pq"])})
    return {"workload": "SegmentationEvaluator reset + update + compute of 8 images, 15 classes, grid-shaped "
                        "segments, dilated thing detections, validation off (the shapes of the reference's recorded "
                        "A100 timings); median of 7 rounds, host clock with device synchronisation",
            "rows": rows,
            "prefix_workload": "segmentation_prefixes of one COCO-like image (133 classes) at the reference's "
                               "recorded sizes, validation off, median of 7 rounds, host clock with device "
                               "synchronisation (result views included, as in the reference's timing)",
            "prefix_rows": prefix_rows}


def panoptic_oracle(arrays):
    """The oracle's PanopticEvaluator over the COCO-shape batches (evaluator.py:291-468 CPU branch)."""
    from oracle import panoptic as opan
    oracle = opan.PanopticOracle(NUM_CLASSES, np.array(isthing(), bool), validate=False)
    for a in arrays:
        oracle.update(a.pred, a.pc, a.gt, a.gc, a.crowd)
    return oracle.compute()


def run_panoptic(args, dev, peak, ours):
    """PanopticEvaluator on COCO-shape batches (B=16, 640 x 640 canvas, images 480-640 per side, 133 classes).

    One step = reset + one update per batch + compute, maps resident in HBM; the
    pair-histogram pass (8 bytes per canvas pixel) is timed on its own stream.
    """
    import torch

    import panoptic_evaluator_gb300 as pe
    from panoptic_evaluator_gb300 import _native, synthetic, tuning
    # The update's launch choices for this shape (101 x 121 slots, 640 x 640 canvas), tuned first.
    tuned = tuning.tune_update(101, 121, 640, 640, images=16, num_classes=NUM_CLASSES, device=dev, repeats=5)
    batches, arrays = [], []
    for k in range(args.panoptic_batches):
        a = synthetic.coco_panoptic_batch(seed=args.seed + 200 + k)
        arrays.append(a)
        batches.append((pe.PanopticBatch(torch.from_numpy(a.pred).to(dev), torch.from_numpy(a.pc).to(dev)),
                        pe.PanopticBatch(torch.from_numpy(a.gt).to(dev), torch.from_numpy(a.gc).to(dev),
                                         torch.from_numpy(a.crowd).to(dev))))
    ev = pe.PanopticEvaluator(NUM_CLASSES, isthing=isthing(), device=dev, validate=False)

    def step():
        ev.reset()
        for p, t in batches:
            ev.update(p, t)
        return ev.compute()["All"]["pq"]

    for _ in range(args.warmup):
        step()
    events, original = [], _native.call

    def timed_call(name, *a):
        if name not in ("pe_update",):
            return original(name, *a)
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        out = original(name, *a)
        e.record()
        events.append((s, e))
        return out

    _native.call = timed_call
    try:
        step()
    finally:
        _native.call = original
    torch.cuda.synchronize()
    steps = max(5, args.steps // 20)
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    start.record()
    for _ in range(steps):
        pq = step()
    end.record()
    end.synchronize()
    ms = start.elapsed_time(end) / steps
    full = ev.compute()
    parity = Parity().compare(full, panoptic_oracle(arrays))
    parity.require("panoptic")
    images = 16 * len(batches)
    ours["panoptic"] = (images / (ms / 1e3), full)
    pixels = sum(int(t.segment_map.numel()) for _, t in batches) // len(batches)
    update_ms = statistics.median(a.elapsed_time(b) for a, b in events)
    achieved = 8 * pixels / (update_ms / 1e3) / 1e9
    return {
        "workload": f"PanopticEvaluator, {len(batches)} COCO-shape batches of 16 images (640 x 640 canvas, images "
                    "480-640 per side, up to 101 target / 121 prediction slots, 133 classes)",
        "value": images / (ms / 1e3), "unit": "images/s", "ms_per_step": ms, "pq": float(pq),
        "parity": parity.summary(f"oracle PanopticEvaluator over all {images} images"),
        "update": {"ms": update_ms, "maps_bytes": 8 * pixels, "effective_gbs": achieved,
                   "note": "one pe_update call of 16 images: pair histogram + scoring + accumulation (3 launches); "
                           "at 52 MB per call launch and scoring latency dominate, not HBM"},
        "update_tuning": {"choice": {"shared_bins": tuned["smem"], "ctas_per_sm": tuned["ctas_per_sm"],
                                     "score_threads": tuned["score_threads"]},
                          "candidates_update_ms": tuned["candidates"],
                          "note": "pe_update timed per launch choice (histogram bins, histogram CTAs per SM, "
                                  "scoring threads) on seeded maps of this shape (tuning.tune_update); the "
                                  "fastest is used for the timing above"},
    }


def run_voronoi(args, dev):
    """PanopticEvaluator on 8 Voronoi images of 256 x 256 (32 slots, 20 classes, 12 things), maps in HBM.

    One step = reset + update + compute, the reference's plain evaluator on its
    CPU-runnable configuration; checked against the oracle.
    """
    import torch

    import panoptic_evaluator_gb300 as pe
    from oracle import panoptic as opan
    from panoptic_evaluator_gb300 import synthetic
    a = synthetic.voronoi_batch(seed=args.seed + 600)
    t = lambda x: torch.from_numpy(x).to(dev)  # noqa: E731
    pred, target = pe.PanopticBatch(t(a.pred), t(a.pc)), pe.PanopticBatch(t(a.gt), t(a.gc), t(a.crowd))
    rows = {}
    for validate in (False, True):
        ev = pe.PanopticEvaluator(a.num_classes, isthing=a.isthing.tolist(), device=dev, validate=validate)

        def step():
            ev.reset()
            ev.update(pred, target)
            return ev.compute()

        for _ in range(max(3, args.warmup)):
            result = step()
        torch.cuda.synchronize()
        steps = max(20, args.steps // 4)
        start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        start.record()
        for _ in range(steps):
            result = step()
        end.record()
        end.synchronize()
        ms = start.elapsed_time(end) / steps
        rows["validate" if validate else "no_validate"] = {"value": 8 / (ms / 1e3), "unit": "images/s",
                                                           "ms_per_step": ms}
    oracle = opan.PanopticOracle(a.num_classes, a.isthing, validate=False)
    oracle.update(a.pred, a.pc, a.gt, a.gc, a.crowd)
    parity = Parity().compare(result, oracle.compute())
    parity.require("voronoi")
    return {"workload": "PanopticEvaluator, 8 Voronoi images of 256 x 256 (24 sites, 32 slots, 20 classes, 12 "
                        "things, 2% crowd, 5% void), perturbed predictions",
            "step": "reset + update + compute, maps resident in HBM", **rows["no_validate"],
            "with_validation": rows["validate"], "pq": float(result["All"]["pq"]),
            "parity": parity.summary("oracle PanopticEvaluator over the 8 images")}, result


def reference_plan(args):
    """Seeds and sizes of the workloads both implementations evaluate (rank 0)."""
    return {"combined_seed": args.seed, "combined_images": args.images, "instance_seed": args.seed + 90,
            "instance_images": args.instance_images, "prefix_seed": args.seed + 300,
            "prefix_images": args.prefix_images, "voronoi_seed": args.seed + 600,
            "panoptic_seed": args.seed + 200, "panoptic_batches": args.panoptic_batches,
            "num_classes": NUM_CLASSES, "things": THINGS, "warmup": 2, "steps": 5}


def run_reference_cuda(args, ours):
    """The reference's own CUDA extension on the same workloads, in a child process (baseline/reference_cuda.py).

    Reports its images/s per workload beside this library's and compares its
    full results with this library's (integers exact, FP64 within PARITY_TOL).
    """
    import tempfile
    recipe = ROOT / "baseline" / "reference_cuda.py"
    extension = ROOT / "baseline" / "_ref" / "panoptic_evaluator" / "_cuda_evaluator.so"
    if not extension.exists():
        return {"unavailable": "the reference's CUDA extension is not built in baseline/_ref "
                               "(baseline/reference_cuda.py stage + build)"}
    with tempfile.TemporaryDirectory() as folder:
        results = Path(folder) / "reference.npz"
        try:
            run = subprocess.run([sys.executable, str(recipe), "measure", "--plan", json.dumps(reference_plan(args)),
                                  "--results", str(results)], capture_output=True, text=True,
                                 timeout=args.reference_cuda_timeout)
        except subprocess.TimeoutExpired:
            return {"unavailable": f"the reference's CUDA run did not finish in {args.reference_cuda_timeout} s"}
        lines = [line for line in run.stdout.splitlines() if line.startswith("{")]
        if run.returncode != 0 or not lines:
            return {"unavailable": "the reference's CUDA run failed: " + (run.stdout + run.stderr)[-600:]}
        line = json.loads(lines[-1])
        reference = dict(np.load(results, allow_pickle=False))
    sys.path.insert(0, str(ROOT / "baseline"))
    import reference_cuda
    for name, row in line["rows"].items():
        if name not in ours:
            continue
        mine = reference_cuda.flatten(ours[name][1], name)
        common = sorted(set(mine) & {k for k in reference if k.startswith(name + "/")})
        parity = Parity().compare({k: mine[k] for k in common}, {k: reference[k] for k in common})
        row["this_library"] = {"value": ours[name][0], "unit": "images/s"}
        row["this_over_reference"] = ours[name][0] / row["value"]
        row["agreement"] = parity.summary("this library's result on the same inputs") | {"keys": len(common)}
    return line


ARM_PARTS = {"0xd4f": "Neoverse V2", "0xd40": "Neoverse V1", "0xd0c": "Neoverse N1", "0xd49": "Neoverse N2",
             "0xd8e": "Neoverse N3", "0xd84": "Neoverse V3"}


def cpu_model():
    """The host CPU's model name (or, on Arm, its implementer part) for the baseline records."""
    import platform
    fields = {}
    try:
        for line in Path("/proc/cpuinfo").read_text().splitlines():
            if ":" in line:
                key, value = (x.strip() for x in line.split(":", 1))
                fields.setdefault(key.lower(), value)
    except OSError:
        pass
    for key in ("model name", "cpu model", "hardware"):
        if key in fields:
            return fields[key]
    part = fields.get("cpu part")
    if part:
        return f"{platform.machine()} {ARM_PARTS.get(part.lower(), 'part ' + part)}"
    return platform.machine()


def cpu_reference_baseline(line):
    """The headline workload's reference CPU number (combined, every host core) in the cpu_baseline form."""
    try:
        row = line["threads_all"]["rows"]["combined"]
    except (KeyError, TypeError):
        return None
    return {"value": row["value"], "unit": "images/s", "cores": line["threads_all"]["threads"], "kind": "reference",
            "sample": row["step"] + f" (torch {line['threads_all']['torch']} on {line['cpu']})"}


def run_reference_cpu(args):
    """The reference's own CPU evaluators (torch, device="cpu") at one thread and at every host core.

    Bounded samples of the C1-C4 workloads (baseline/reference_cuda.py measure-cpu), each in a child
    process so that its torch thread count is its own.
    """
    recipe = ROOT / "baseline" / "reference_cuda.py"
    if not (ROOT / "baseline" / "_ref" / "panoptic_evaluator" / "__init__.py").exists():
        return {"unavailable": "the reference package is not staged in baseline/_ref"}
    plan = {"voronoi_seed": args.seed + 600, "panoptic_seed": args.seed + 200, "instance_seed": args.seed + 90,
            "combined_seed": args.seed, "num_classes": NUM_CLASSES, "things": THINGS, "instance_sample": 2,
            "combined_sample": 8, "rounds": 3}
    out = {"kind": "reference", "cpu": cpu_model(), "host_cores": os.cpu_count()}
    for label, threads in (("threads_1", 1), ("threads_all", os.cpu_count() or 1)):
        try:
            run = subprocess.run([sys.executable, str(recipe), "measure-cpu", "--plan", json.dumps(plan),
                                  "--threads", str(threads)], capture_output=True, text=True, timeout=300)
            lines = [line for line in run.stdout.splitlines() if line.startswith("{")]
            out[label] = json.loads(lines[-1]) if run.returncode == 0 and lines else \
                {"unavailable": (run.stdout + run.stderr)[-400:]}
        except subprocess.TimeoutExpired:
            out[label] = {"unavailable": "did not finish in 300 s"}
    return out


def isthing():
    return [c < THINGS for c in range(NUM_CLASSES)]


def oracle_args(img):
    return (img.pred, img.pred_classes, img.det_masks, img.det_classes, img.scores, img.target, img.target_classes,
            img.crowd, NUM_CLASSES, isthing())


def oracle_step(images, pool=None):
    from oracle import combined as ocomb
    work = [oracle_args(i) for i in images]
    parts = pool.map(ocomb.image_update, work) if pool is not None else [ocomb.image_update(w) for w in work]
    return ocomb.merge(parts, NUM_CLASSES, isthing()).compute()


class Clocks:
    """Sample SM clocks and throttle reasons with nvidia-smi while the timed region runs."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None

    def __enter__(self):
        exe = shutil.which("nvidia-smi")
        if exe:
            self.proc = subprocess.Popen([exe, "-i", str(self.index), f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [line for line in out.splitlines() if line.strip()]

    def summary(self):
        rows = []
        for line in getattr(self, "lines", []):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), parts[5:9]))
            except ValueError:
                continue
        if not rows:
            return None
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        reasons = sorted({names[i] for _, _, flags in rows for i, f in enumerate(flags) if f.lower() == "active"})
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows)}


def measured_peak():
    path = ROOT / "MEASURED_PEAKS.json"
    if path.exists():
        data = json.loads(path.read_text())
        return float(data["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def traffic_ratio():
    """DRAM bytes per algorithmic byte of the fused pass, from the committed ncu summary (if any)."""
    path = ROOT / "profiles" / "seg_pass_traffic.txt"
    if not path.exists():
        return None
    for line in path.read_text().splitlines():
        if line.startswith("dram_bytes_per_algorithmic_byte:"):
            return float(line.split(":", 1)[1])
    return None


def _reference_worker(conn, seed, indices):
    """Own a fixed partition of the workload: generate it once, then evaluate it per step."""
    from oracle import combined as ocomb
    from panoptic_evaluator_gb300 import synthetic
    images = [synthetic.segmentation_one(seed, i) for i in indices]
    conn.send("ready")
    while True:
        message = conn.recv()
        if message == "stop":
            break
        count = message[1]  # ("step", images of the partition to evaluate)
        parts = [ocomb.image_update(oracle_args(img)) for img in images[:count]]
        conn.send(ocomb.merge(parts, NUM_CLASSES, isthing()))
    conn.close()


def run_reference(args):
    """The reference algorithm's CPU implementation (numpy oracle) on all host cores."""
    rank, world, _ = rank_info()
    if rank != 0:
        return
    from oracle import combined as ocomb
    cores = os.cpu_count() or 1
    workers = max(1, min(cores, args.images))
    ctx = mp.get_context("spawn")
    procs, conns = [], []
    for k in range(workers):
        parent, child = ctx.Pipe()
        proc = ctx.Process(target=_reference_worker, args=(child, args.seed, list(range(k, args.images, workers))),
                           daemon=True)
        proc.start()
        procs.append(proc)
        conns.append(parent)
    for c in conns:
        assert c.recv() == "ready"

    partition = len(range(0, args.images, workers))  # images per worker (the first worker's share)

    def step(count):
        for c in conns:
            c.send(("step", count))
        parts = [c.recv() for c in conns]
        return ocomb.merge(parts, NUM_CLASSES, isthing()).compute()

    t0 = time.perf_counter()
    step(partition)  # first warm-up step over the whole workload, also sizes the per-step sample
    first = time.perf_counter() - t0
    # Keep the timed run near 90 s for any --steps: every worker stays busy but evaluates only the first
    # `count` images of its partition per step when the whole workload is too slow (images/s is a
    # per-image rate either way).
    count = max(1, min(partition, int(partition * 90.0 / max(first * args.steps, 1e-9))))
    sample = sum(min(count, len(range(k, args.images, workers))) for k in range(workers))

    def step_sample():
        return step(count)

    for _ in range(max(0, args.warmup - 1)):
        step_sample()
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        step_sample()
        times.append(time.perf_counter() - t0)
    for c in conns:
        c.send("stop")
    for proc in procs:
        proc.join(timeout=10)
    ms = 1000 * statistics.mean(times)
    value = sample / (ms / 1000)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "images/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int64 counts, f64 metrics (numpy)", "data": "synthetic",
        "config": {"workload": WORKLOAD, "images": args.images, "step": "update of every image + compute"},
        "cpu_baseline": {"value": value, "unit": "images/s", "cores": workers, "kind": "port",
                         "sample": f"{sample} of the {args.images} workload images per step (update + compute), "
                                   f"{workers} worker processes each owning a fixed partition"},
        "e2e": {"value": value, "unit": "images/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def headline(result):
    import torch
    inst = result["instance"]
    return torch.stack([result["All"]["pq"], result["Things"]["pq"], result["Stuff"]["pq"], result["miou"],
                        inst["ap"], inst["ap50"], inst["ap75"], inst["ar100"]])


def run_case(args):
    """A few steps of one workload at a chosen size, for profiler captures (prints one summary line)."""
    ctx = mp.get_context("spawn")
    with ctx.Pool(min(16, os.cpu_count() or 1)) as pool:  # started before any CUDA call
        if args.case == "combined":
            from panoptic_evaluator_gb300 import synthetic
            images = synthetic.segmentation_batch(seed=args.seed, images=args.case_images, pool=pool)
        elif args.case == "panoptic":
            images = None
        elif args.case == "prefix":
            args.prefix_images = args.case_images
            images = generate_prefix(args, pool)
        else:
            args.instance_images = args.case_images
            images = generate_instance(args, pool)
    import torch

    import panoptic_evaluator_gb300 as pe
    dev = torch.device("cuda", 0)
    if args.case == "prefix":
        target = pe.PanopticBatch(torch.from_numpy(np.stack([i.target for i in images])).to(dev),
                                  torch.from_numpy(np.stack([i.target_classes for i in images])).to(dev),
                                  torch.from_numpy(np.stack([i.crowd for i in images])).to(dev))
        pred = pe.InstanceBatch([torch.from_numpy(i.masks).to(dev) for i in images],
                                [torch.from_numpy(i.classes).to(dev) for i in images])

        def step():
            result = pe.segmentation_prefixes(pred, target, NUM_CLASSES, isthing=isthing(),
                                              checkpoints=list(range(8, 65, 8)), validate=False)
            return result[0][-1]["All"]["pq"]
    elif args.case == "panoptic":
        from panoptic_evaluator_gb300 import synthetic
        batches = []
        for k in range(max(1, args.case_images // 16)):
            a = synthetic.coco_panoptic_batch(seed=args.seed + 200 + k)
            batches.append((pe.PanopticBatch(torch.from_numpy(a.pred).to(dev), torch.from_numpy(a.pc).to(dev)),
                            pe.PanopticBatch(torch.from_numpy(a.gt).to(dev), torch.from_numpy(a.gc).to(dev),
                                             torch.from_numpy(a.crowd).to(dev))))
        images = [None] * (16 * len(batches))
        ev = pe.PanopticEvaluator(NUM_CLASSES, isthing=isthing(), device=dev, validate=False)

        def step():
            ev.reset()
            for p, t in batches:
                ev.update(p, t)
            return ev.compute()["All"]["pq"]
    elif args.case == "combined":
        from panoptic_evaluator_gb300.ragged import SegmentationImages
        arena = SegmentationImages([i.target for i in images], [i.target_classes for i in images],
                                   [i.crowd for i in images], [i.pred for i in images],
                                   [i.pred_classes for i in images], [i.det_masks for i in images],
                                   [i.det_classes for i in images], [i.scores for i in images], device=dev)
        ev = pe.SegmentationEvaluator(NUM_CLASSES, isthing=isthing(), device=dev, validate=False)

        def step():
            ev.reset()
            ev.update_images(arena)
            return ev.compute()["All"]["pq"]
    else:
        pred = pe.InstanceBatch([torch.from_numpy(i.pred_masks).to(dev) for i in images],
                                [torch.from_numpy(i.pred_classes).to(dev) for i in images],
                                [torch.from_numpy(i.scores).to(dev) for i in images])
        target = pe.InstanceBatch([torch.from_numpy(i.gt_masks).to(dev) for i in images],
                                  [torch.from_numpy(i.gt_classes).to(dev) for i in images],
                                  crowd=[torch.from_numpy(i.crowd).to(dev) for i in images])
        ev = pe.InstanceEvaluator(80, device=dev, validate=False)

        def step():
            ev.reset()
            ev.update(pred, target)
            return ev.compute()["ap"]
    for _ in range(args.case_steps):
        value = step()
    torch.cuda.synchronize()
    print(f"case {args.case}: {len(images)} images, {args.case_steps} steps, result {float(value):.12f}", flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    if args.case:
        run_case(args)
        return
    rank, world, local = rank_info()
    ctx = mp.get_context("spawn")
    with ctx.Pool(min(16, os.cpu_count() or 1)) as pool:  # started before any CUDA call
        images = generate(args, rank, pool)
        serving = generate_serving(args, pool) if args.serve_requests and world == 1 else None
        instance_images = generate_instance(args, pool) if args.instance_images and world == 1 else None
        prefix_images = generate_prefix(args, pool) if args.prefix_images and world == 1 else None
        # The oracle's results for every section's whole workload, computed here in parallel: each
        # section compares its GPU result with them (integers exact, FP64 within PARITY_TOL).
        expected = oracle_step(images, pool)
        serving_expected = serving_oracles(*serving, pool) if serving is not None else None
        instance_expected = instance_oracle(instance_images, pool) if instance_images else None
        prefix_expected = pool.map(_prefix_oracle, prefix_images, chunksize=1) if prefix_images else None
    import torch
    import torch.distributed as dist

    import panoptic_evaluator_gb300 as pe
    from panoptic_evaluator_gb300 import _native, combined
    from panoptic_evaluator_gb300.ragged import SegmentationImages

    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    dev = torch.device("cuda", local)
    arena = SegmentationImages([i.target for i in images], [i.target_classes for i in images],
                               [i.crowd for i in images], [i.pred for i in images], [i.pred_classes for i in images],
                               [i.det_masks for i in images], [i.det_classes for i in images],
                               [i.scores for i in images], device=dev)
    torch.cuda.synchronize()
    ev = pe.SegmentationEvaluator(NUM_CLASSES, isthing=isthing(), device=dev, validate=False)

    def step():
        ev.reset()
        ev.update_images(arena)
        return headline(ev.compute())

    # The fused pass's launch choices (chunks per counter grab, CTAs per SM) tuned on this batch first.
    from panoptic_evaluator_gb300 import tuning
    pass_tuning = tuning.tune_pass(ev, arena, repeats=3)
    # Warm-up (eager), counting this library's launches per step.
    for _ in range(max(1, args.warmup)):
        step()
    torch.cuda.synchronize()
    before = _native.launch_count()
    step()
    torch.cuda.synchronize()
    launches_per_step = _native.launch_count() - before

    # Dominant kernel (the fused pixel pass) timed alone with events on its stream.
    stream = torch.cuda.current_stream(dev)
    pass_ms = []
    combined.PASS_EVENTS = []
    for _ in range(3):
        step()
    torch.cuda.synchronize()
    pass_ms = [s.elapsed_time(e) for s, e in combined.PASS_EVENTS]
    combined.PASS_EVENTS = None

    # CUDA graph of the whole step.
    graph = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream(dev)
    side.wait_stream(stream)
    with torch.cuda.stream(side):
        step()
    stream.wait_stream(side)
    with torch.cuda.graph(graph):
        out = step()
    for _ in range(args.warmup):
        graph.replay()
    torch.cuda.synchronize()

    def timed(fn, steps):
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()
        start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        start.record()
        for _ in range(steps):
            fn()
        end.record()
        end.synchronize()
        ms = start.elapsed_time(end) / steps
        if world > 1:
            t = torch.tensor([ms], device=dev)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            ms = float(t.item())
        return ms

    index = os.environ.get("CUDA_VISIBLE_DEVICES", str(local)).split(",")[local] if world == 1 or \
        "CUDA_VISIBLE_DEVICES" in os.environ else str(local)
    with Clocks(index if index.isdigit() else local) as clocks:
        ms_graph = timed(graph.replay, args.steps)
    result_dev = out.clone()

    # End to end: upload the pinned host arena, replay, read the headline metrics back.
    host_out = torch.empty(out.shape, dtype=out.dtype, pin_memory=True)

    def e2e_step():
        arena.upload()
        graph.replay()
        host_out.copy_(out, non_blocking=True)
        torch.cuda.current_stream(dev).synchronize()

    for _ in range(2):
        e2e_step()
    ms_e2e = timed(e2e_step, max(2, args.steps // 2))

    # Plain path: the reference-style per-image update (B = 1 per call) on the same GPU.
    plain_images = [(torch.from_numpy(i.target[None]).to(dev), torch.from_numpy(i.target_classes[None]).to(dev),
                     torch.from_numpy(i.crowd[None]).to(dev), torch.from_numpy(i.pred[None]).to(dev),
                     torch.from_numpy(i.pred_classes[None]).to(dev), torch.from_numpy(i.det_masks).to(dev),
                     torch.from_numpy(i.det_classes).to(dev), torch.from_numpy(i.scores).to(dev)) for i in images]
    plain = pe.SegmentationEvaluator(NUM_CLASSES, isthing=isthing(), device=dev, validate=False)

    def plain_step():
        plain.reset()
        for t, tc, cr, p, pc, m, dc, sc in plain_images:
            plain.update(pe.PanopticBatch(p, pc), pe.InstanceBatch([m], [dc], [sc]), pe.PanopticBatch(t, tc, cr))
        return headline(plain.compute())

    plain_out = plain_step()
    torch.cuda.synchronize()
    ms_plain = timed(plain_step, args.plain_steps)
    torch.testing.assert_close(plain_step(), result_dev, rtol=1e-12, atol=1e-12)
    # The whole result of the batched path (the graph's kernels, run eagerly once more) against the oracle.
    ev.reset()
    ev.update_images(arena)
    full = ev.compute()
    parity = Parity().compare(full, expected)
    parity.require("headline")

    n_images = args.images * world
    value = n_images / (ms_graph / 1000)
    if rank != 0:
        dist.destroy_process_group()
        return
    ours = {"combined": (value, full)}
    voronoi_line = None
    if world == 1:
        voronoi_line, voronoi_result = run_voronoi(args, dev)
        ours["voronoi"] = (voronoi_line["value"], voronoi_result)
    serving_line = run_serving(args, *serving, dev, serving_expected) if serving is not None else None
    instance_line = (run_instance(args, instance_images, dev, measured_peak()[0], instance_expected, ours)
                     if instance_images else None)
    panoptic_line = (run_panoptic(args, dev, measured_peak()[0], ours)
                     if args.panoptic_batches and world == 1 else None)
    published_line = run_published(args, dev) if args.published and world == 1 else None
    prefix_line = (run_prefix(args, prefix_images, dev, measured_peak()[0], prefix_expected, ours)
                   if prefix_images else None)
    reference_cuda_line = run_reference_cuda(args, ours) if args.reference_cuda and world == 1 else None
    reference_cpu_line = run_reference_cpu(args) if args.reference_cpu and world == 1 else None
    # CPU baseline: the numpy oracle on a bounded sample, one process, after the GPU work.
    sample = images[: args.cpu_sample]
    t0 = time.perf_counter()
    oracle_step(sample)
    cpu_s = time.perf_counter() - t0
    peak, peak_kind = measured_peak()
    algo_bytes = arena.algorithmic_bytes()
    pass_time = statistics.median(pass_ms) / 1000
    achieved = algo_bytes / pass_time / 1e9
    ratio = traffic_ratio()
    line = {
        "metric": METRIC, "value": value, "unit": "images/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_graph, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32 counts from int32 maps + u8 masks; f64 metrics", "data": "synthetic",
        "config": {"workload": WORKLOAD, "images": args.images, "mode": "batched: 1 descriptor table, CUDA graph of "
                   "reset+update+compute", "l2": "inputs larger than L2 (arena %.2f GB per step)" % (arena.nbytes / 1e9),
                   "mean_pixels": float(arena.hw.mean()), "mean_detections": float(arena.D.mean())},
        "plain": {"value": n_images / (ms_plain / 1000), "unit": "images/s", "ms_per_step": ms_plain,
                  "mode": "per-image update() calls (B=1) through the same kernels"},
        "batched_vs_plain": ms_plain / ms_graph,
        "pass_tuning": {"choice": {"chunks_per_grab": pass_tuning["grab"], "ctas_per_sm": pass_tuning["ctas_per_sm"]},
                        "candidates_pass_ms": pass_tuning["candidates"],
                        "note": "fused pass timed per launch choice on this batch (tuning.tune_pass); the fastest "
                                "is used for every timing above"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_kind": peak_kind, "kernel": "seg_pass_kernel",
                     "algorithmic_bytes_per_launch": algo_bytes, "kernel_ms": pass_time * 1000,
                     "traffic": None if ratio is None else ratio * algo_bytes},
        "cpu_baseline": {"value": len(sample) / cpu_s, "unit": "images/s", "cores": 1, "kind": "port",
                         "sample": f"{len(sample)} images of the workload through the numpy oracle, one process"},
        "cpu_baseline_reference": cpu_reference_baseline(reference_cpu_line),
        "e2e": {"value": n_images / (ms_e2e / 1000), "unit": "images/s", "ms_per_step": ms_e2e,
                "h2d_bytes_per_step": arena.nbytes, "d2h_bytes_per_step": int(out.numel() * out.element_size())},
        "gpu_launches": int(launches_per_step * args.steps),
        "clocks": clocks.summary(),
        "headline_metrics": [float(x) for x in result_dev.cpu()],
        "parity": parity.summary(f"oracle SegmentationEvaluator over all {args.images} images (per rank)"),
        "voronoi": voronoi_line,
        "reference_cuda": reference_cuda_line,
        "reference_cpu": reference_cpu_line,
        "serving": serving_line,
        "instance": instance_line,
        "panoptic": panoptic_line,
        "prefix": prefix_line,
        "published_shapes": published_line,
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
