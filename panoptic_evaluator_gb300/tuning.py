"""Autotuner of the per-call update, the batched fused pass and the mask contraction's CTA split.

The launch choices of ``PanopticEvaluator.update``'s kernels, histogram bins in
shared or global memory, histogram CTAs per SM, and threads of each image's
scoring CTA, are kept in the library per bucket of (floor(log2(G * P)),
floor(log2(pixels per image))) (``pe_tune_update``). ``tune_update`` times the
candidates on seeded maps of the caller's shape through the public API, keeps
the fastest for that bucket, and can persist it to a JSON cache that ``load``
(or the ``PE_GB300_TUNING`` environment variable, read when the library loads)
applies in later processes. Every choice computes the same counts: only speed
differs. The reference instead reads ``PANOPTIC_HISTOGRAM`` and
``PANOPTIC_SCORING`` on every call (histogram_kernel.cu:240-246,309-310).

The batched fused pass (``SegmentationEvaluator.update_images``) takes its
8192-pixel chunks from a device counter; ``tune_pass`` times how many chunks a
producer takes per grab (1, 2, 4) and the CTAs per SM (1, 2) on the caller's
own batch and keeps the fastest for that batch size (``pe_tune_pass``), in the
same JSON cache.

The mask contraction (``InstanceEvaluator.update``) splits a batch into
contiguous CTA ranges of equal cost, where a block loaded by TMA counts a
fraction of a staged one; ``tune_contract`` times that weight on the caller's
batch per bucket of the share of mask bytes TMA loads, also in the cache.
"""

from __future__ import annotations

import ctypes
import json
import math
import os
import statistics
from pathlib import Path

import numpy as np
import torch

from . import _native as N

MAX_SMEM_BINS = 50 * 1024  # G * P bins that fit in shared memory (the kernel's kMaxSmemBins)
CTAS_PER_SM = (1, 2, 4)
SCORE_THREADS = (256, 512, 1024)
KEYS = ("bins_bucket", "pixels_bucket", "smem", "ctas_per_sm", "score_threads")


def bucket(bins: int, pixels: int) -> tuple[int, int]:
    """The library's tuning key for a launch of G * P = bins and `pixels` per image."""
    return int(math.floor(math.log2(bins))), int(math.floor(math.log2(pixels)))


def cache_path(path=None) -> Path:
    return Path(path or os.environ.get("PE_GB300_TUNING") or Path.home() / ".cache" / "pe_gb300" / "update.json")


def register(bins_bucket: int, pixels_bucket: int, smem: int, ctas_per_sm: int, score_threads: int) -> None:
    N.call("pe_tune_update", 1 << bins_bucket, 1 << pixels_bucket, int(smem), int(ctas_per_sm), int(score_threads))


def forget(bins_bucket: int, pixels_bucket: int) -> None:
    """Remove a bucket's entry: the built-in rule applies again."""
    N.call("pe_tune_update", 1 << bins_bucket, 1 << pixels_bucket, -1, 1, 256)


def choice(bins: int, pixels: int) -> tuple[int, int, int]:
    """(shared bins, histogram CTAs per SM, scoring threads) a launch of this shape uses now."""
    smem, per_sm, threads = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
    N.call("pe_update_choice", int(bins), int(pixels), ctypes.byref(smem), ctypes.byref(per_sm),
           ctypes.byref(threads))
    return smem.value, per_sm.value, threads.value


def read(path=None) -> list[dict]:
    p = cache_path(path)
    if not p.exists():
        return []
    return [e for e in json.loads(p.read_text()).get("update", []) if set(KEYS) <= set(e)]


def write(entries: list[dict], path=None) -> Path:
    """Merge entries into the cache file (one per bucket, the newest wins)."""
    p = cache_path(path)
    data = json.loads(p.read_text()) if p.exists() else {}
    merged = {(e["bins_bucket"], e["pixels_bucket"]): {k: e[k] for k in KEYS} for e in read(p) + list(entries)}
    data["update"] = sorted(merged.values(), key=lambda e: (e["bins_bucket"], e["pixels_bucket"]))
    p.parent.mkdir(parents=True, exist_ok=True)
    p.write_text(json.dumps(data, indent=1))
    return p


def load(path=None) -> int:
    """Register every cached choice in the library; returns how many."""
    entries = read(path)
    for e in entries:
        register(*(e[k] for k in KEYS))
    passes = read_pass(path)
    for e in passes:
        register_pass(*(e[k] for k in PASS_KEYS))
    contracts = read_contract(path)
    for e in contracts:
        register_contract(*(e[k] for k in CONTRACT_KEYS))
    return len(entries) + len(passes) + len(contracts)


def _maps(rng, images, height, width, slots, block):
    """Slot maps of rectangular segments of about `block` pixels a side, slots 0..slots-1 (0 = void)."""
    rows, cols = -(-height // block), -(-width // block)
    cells = rng.integers(0, slots, (images, rows, cols)).astype(np.int32)
    return np.repeat(np.repeat(cells, block, 1), block, 2)[:, :height, :width].copy()


def tune_update(G: int, P: int, height: int, width: int, *, images: int = 16, num_classes: int = 133,
                device=None, repeats: int = 7, persist: bool = False, path=None, seed: int = 0) -> dict:
    """Time the update's launch choices for this shape, keep and return the fastest.

    G / P: target / prediction slots per image (slot 0 void), `images` per update. The timed call is
    ``PanopticEvaluator.update`` (CUDA events on its stream, median of `repeats`). The histogram
    choices are timed first with the built-in scoring block, then the scoring blocks with the best
    histogram choice.
    """
    from .evaluator import PanopticBatch, PanopticEvaluator
    dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
    rng = np.random.default_rng(seed)
    side = max(8, int(math.sqrt(height * width / max(G, P))))
    gt = torch.from_numpy(_maps(rng, images, height, width, G, side)).to(dev)
    pr = torch.from_numpy(_maps(rng, images, height, width, P, max(4, side // 2))).to(dev)
    gc = torch.from_numpy(rng.integers(0, num_classes, (images, G)).astype(np.int32)).to(dev)
    pc = torch.from_numpy(rng.integers(0, num_classes, (images, P)).astype(np.int32)).to(dev)
    gc[:, 0] = -1
    pc[:, 0] = -1
    target, prediction = PanopticBatch(gt, gc), PanopticBatch(pr, pc)
    key = bucket(G * P, height * width)
    evaluator = PanopticEvaluator(num_classes, device=dev, validate=False)
    stream = torch.cuda.current_stream(dev)

    def timed(smem, per_sm, threads):
        register(*key, smem, per_sm, threads)
        times = []
        for i in range(repeats + 2):
            start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            start.record(stream)
            evaluator.update(prediction, target)
            end.record(stream)
            end.synchronize()
            if i >= 2:
                times.append(start.elapsed_time(end))
        return {"smem": smem, "ctas_per_sm": per_sm, "score_threads": threads, "ms": statistics.median(times)}

    try:
        first = [timed(s, c, SCORE_THREADS[0]) for s in ((1, 0) if G * P <= MAX_SMEM_BINS else (0,))
                 for c in CTAS_PER_SM]
        best = min(first, key=lambda r: r["ms"])
        second = [timed(best["smem"], best["ctas_per_sm"], t) for t in SCORE_THREADS[1:]]
    except BaseException:
        forget(*key)  # leave the built-in rule in place
        raise
    results = first + second
    best = min(results, key=lambda r: r["ms"])
    register(*key, best["smem"], best["ctas_per_sm"], best["score_threads"])
    entry = {"bins_bucket": key[0], "pixels_bucket": key[1], "smem": best["smem"],
             "ctas_per_sm": best["ctas_per_sm"], "score_threads": best["score_threads"]}
    if persist:
        write([entry], path)
    return {**entry, "ms": best["ms"], "candidates": results}


# ---- the batched fused pass ----------------------------------------------------

PASS_GRABS = (1, 2, 4)
PASS_CTAS_PER_SM = (1, 2)
PASS_KEYS = ("chunks_bucket", "grab", "ctas_per_sm")


def register_pass(chunks_bucket: int, grab: int, ctas_per_sm: int) -> None:
    N.call("pe_tune_pass", 1 << chunks_bucket, int(grab), int(ctas_per_sm))


def forget_pass(chunks_bucket: int) -> None:
    N.call("pe_tune_pass", 1 << chunks_bucket, -1, 1)


def pass_choice(chunks: int) -> tuple[int, int]:
    """(chunks per counter grab, CTAs per SM) a batched pass over `chunks` 8192-pixel chunks uses now."""
    grab, per_sm = ctypes.c_int32(), ctypes.c_int32()
    N.call("pe_pass_choice", int(chunks), ctypes.byref(grab), ctypes.byref(per_sm))
    return grab.value, per_sm.value


def tune_pass(evaluator, images, *, repeats: int = 5, persist: bool = False, path=None) -> dict:
    """Time the fused pass's launch choices on a batch, keep and return the fastest.

    `evaluator` is a SegmentationEvaluator and `images` a ragged batch
    (``ragged.SegmentationImages``) on its device. Each candidate (chunks per
    counter grab x CTAs per SM) runs ``update_images`` `repeats` times after a
    warm-up; the fused pass is timed with CUDA events on its stream (median).
    The evaluator is reset afterwards. Every choice gives the same counts: only
    the order in which CTAs take chunks differs.
    """
    from . import combined
    chunks = images.table(evaluator.instance._scratch).total_chunks
    if not chunks:
        raise ValueError("the batch has no pixels to tune on")
    key = int(math.floor(math.log2(chunks)))
    results = []
    saved = combined.PASS_EVENTS
    try:
        for grab in PASS_GRABS:
            for per_sm in PASS_CTAS_PER_SM:
                register_pass(key, grab, per_sm)
                combined.PASS_EVENTS = []
                for _ in range(repeats + 1):
                    evaluator.update_images(images)
                torch.cuda.synchronize(evaluator.device)
                times = [s.elapsed_time(e) for s, e in combined.PASS_EVENTS[1:]]
                results.append({"grab": grab, "ctas_per_sm": per_sm, "ms": statistics.median(times)})
    except BaseException:
        forget_pass(key)
        raise
    finally:
        combined.PASS_EVENTS = saved
        evaluator.reset()
    best = min(results, key=lambda r: r["ms"])
    register_pass(key, best["grab"], best["ctas_per_sm"])
    entry = {"chunks_bucket": key, "grab": best["grab"], "ctas_per_sm": best["ctas_per_sm"]}
    if persist:
        write_pass([entry], path)
    return {**entry, "ms": best["ms"], "candidates": results}


def read_pass(path=None) -> list[dict]:
    p = cache_path(path)
    if not p.exists():
        return []
    return [e for e in json.loads(p.read_text()).get("pass", []) if set(PASS_KEYS) <= set(e)]


def write_pass(entries: list[dict], path=None) -> Path:
    """Merge pass entries into the cache file (one per bucket, the newest wins); update entries are kept."""
    p = cache_path(path)
    data = json.loads(p.read_text()) if p.exists() else {}
    merged = {e["chunks_bucket"]: {k: e[k] for k in PASS_KEYS} for e in read_pass(p) + list(entries)}
    data["pass"] = sorted(merged.values(), key=lambda e: e["chunks_bucket"])
    p.parent.mkdir(parents=True, exist_ok=True)
    p.write_text(json.dumps(data, indent=1))
    return p


# ---- the mask contraction's CTA split ---------------------------------------------
# A batch mixing images loaded by TMA (16-byte mask rows) with staged images is split
# into contiguous CTA ranges of equal cost, a TMA block counting `tma_cost` of a staged
# one. The best weight depends on the mix, so it is kept per bucket of the fraction of
# mask bytes that TMA loads (tenths). Every weight gives the same counts.

CONTRACT_TMA_COSTS = (0.45, 0.6, 0.73, 0.85, 1.0, 1.2)
CONTRACT_KEYS = ("tma_bucket", "tma_cost")
_contract_costs: dict[int, float] = {}


def contract_bucket(dets, gts, pixels, tma) -> int:
    """Tenths (0-10) of a batch's mask bytes, (D + G) x H x W per image, on images loaded by TMA."""
    dets, gts, pixels = (np.asarray(x, np.int64).reshape(-1) for x in (dets, gts, pixels))
    mask_bytes = (dets + gts) * pixels
    total = int(mask_bytes.sum())
    return int(10 * int(mask_bytes[np.asarray(tma, bool).reshape(-1)].sum()) // total) if total else 0


def register_contract(tma_bucket: int, tma_cost: float) -> None:
    _contract_costs[int(tma_bucket)] = float(tma_cost)


def forget_contract(tma_bucket: int) -> None:
    _contract_costs.pop(int(tma_bucket), None)


def contract_cost(tma_bucket: int) -> float:
    """The TMA block weight a batch in this bucket uses now (the built-in CONTRACT_TMA_COST without an entry)."""
    from ._batch import CONTRACT_TMA_COST
    return _contract_costs.get(int(tma_bucket), CONTRACT_TMA_COST)


def tune_contract(evaluator, prediction, target, *, repeats: int = 5, persist: bool = False, path=None) -> dict:
    """Time the contraction's CTA split weights on a batch, keep and return the fastest.

    `evaluator` is an InstanceEvaluator and `prediction` / `target` an update's
    InstanceBatch pair on its device. For each weight in CONTRACT_TMA_COSTS the
    update runs `repeats` times after a warm-up and `pe_inst_contract` is timed
    with CUDA events on its stream (median). The evaluator is reset afterwards.
    """
    from . import instance
    pm = [m.contiguous() for m in prediction.masks]
    gm = [m.contiguous() for m in target.masks]
    dets = np.array([m.shape[0] for m in pm], np.int64)
    gts = np.array([m.shape[0] for m in gm], np.int64)
    pixels = np.array([m.shape[1] * m.shape[2] for m in pm], np.int64)
    flags = instance.mask_flags([m.data_ptr() for m in pm], [m.data_ptr() for m in gm], pixels)
    tma = ((flags & 2) != 0) & (dets > 0) & (gts > 0) & (pixels > 0) & instance.DIRECT_CONTRACTION
    key = contract_bucket(dets, gts, pixels, tma)
    events = []
    original = N.call

    def timed(name, *args):
        if name != "pe_inst_contract":
            return original(name, *args)
        start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        start.record()
        out = original(name, *args)
        end.record()
        events.append((start, end))
        return out

    results = []
    try:
        for cost in CONTRACT_TMA_COSTS:
            register_contract(key, cost)
            events.clear()
            N.call = timed
            try:
                for _ in range(repeats + 1):
                    evaluator.update(prediction, target)
            finally:
                N.call = original
            torch.cuda.synchronize(evaluator.device)
            results.append({"tma_cost": cost, "ms": statistics.median(s.elapsed_time(e) for s, e in events[1:])})
    except BaseException:
        forget_contract(key)
        raise
    finally:
        evaluator.reset()
    best = min(results, key=lambda r: r["ms"])
    register_contract(key, best["tma_cost"])
    entry = {"tma_bucket": key, "tma_cost": best["tma_cost"]}
    if persist:
        write_contract([entry], path)
    return {**entry, "ms": best["ms"], "candidates": results}


def read_contract(path=None) -> list[dict]:
    p = cache_path(path)
    if not p.exists():
        return []
    return [e for e in json.loads(p.read_text()).get("contract", []) if set(CONTRACT_KEYS) <= set(e)]


def write_contract(entries: list[dict], path=None) -> Path:
    """Merge contraction entries into the cache file (one per bucket, the newest wins); other entries are kept."""
    p = cache_path(path)
    data = json.loads(p.read_text()) if p.exists() else {}
    merged = {e["tma_bucket"]: {k: e[k] for k in CONTRACT_KEYS} for e in read_contract(p) + list(entries)}
    data["contract"] = sorted(merged.values(), key=lambda e: e["tma_bucket"])
    p.parent.mkdir(parents=True, exist_ok=True)
    p.write_text(json.dumps(data, indent=1))
    return p
