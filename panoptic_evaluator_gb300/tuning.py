"""Autotuner of the per-call update (pair histogram + per-image scoring).

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
    merged = {(e["bins_bucket"], e["pixels_bucket"]): {k: e[k] for k in KEYS} for e in read(p) + list(entries)}
    p.parent.mkdir(parents=True, exist_ok=True)
    p.write_text(json.dumps({"update": sorted(merged.values(), key=lambda e: (e["bins_bucket"],
                                                                            e["pixels_bucket"]))}, indent=1))
    return p


def load(path=None) -> int:
    """Register every cached choice in the library; returns how many."""
    entries = read(path)
    for e in entries:
        register(*(e[k] for k in KEYS))
    return len(entries)


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
