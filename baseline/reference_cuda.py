"""Recipe: the reference's own CUDA extension, for timing beside this library and for drop-in tests.

MEASUREMENT / TEST INFRASTRUCTURE ONLY. Nothing in ``panoptic_evaluator_gb300``
imports it. It handles AndyBarcia/panoptic-evaluator's unmodified package
(``panoptic_evaluator/*.py``, its ``csrc/`` extension and ``tests/``) in the
git-ignored folder ``baseline/_ref/``:

``stage --reference <checkout>``
    copies the package and its tests from a reference checkout into
    ``baseline/_ref/`` (sources are never committed; the folder travels with
    the working tree to a GPU machine, which has no checkout and cannot run
    binaries built on another architecture).
``build``
    compiles the reference's extension as its ``setup.py`` declares it
    (``csrc/bindings.cpp`` + the four ``*_kernel.cu``, ``-O3``) for sm_103 with
    ``torch.utils.cpp_extension`` into
    ``baseline/_ref/panoptic_evaluator/_cuda_evaluator.so``. The reference's
    kernels are generic CUDA, so they get the plain ``sm_103`` target.

    python baseline/reference_cuda.py stage --reference <path to the reference checkout>
    python baseline/reference_cuda.py build

``measure --plan <json> --results <npz>``
    times the reference's evaluators on CUDA (its public API, its own
    extension, inputs resident on the device) over the seeded synthetic
    workloads the plan names, prints one JSON line of timings and writes the
    full results for comparison. ``bench.py`` runs it in a child process.

``measure-cpu --plan <json> --threads <k>``
    times the reference's CPU evaluators (torch on the host, ``device="cpu"``)
    on bounded samples of the same workloads with ``torch.set_num_threads(k)``.

``load()`` imports the staged package with its own extension and checks that
the extension module really is the one built here.
"""

from __future__ import annotations

import argparse
import importlib
import os
import platform
import shutil
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
STAGE = HERE / "_ref"
PACKAGE = STAGE / "panoptic_evaluator"
EXTENSION = PACKAGE / "_cuda_evaluator.so"
SOURCES = ("csrc/bindings.cpp", "csrc/histogram_kernel.cu", "csrc/compute_kernel.cu", "csrc/instance_kernel.cu",
           "csrc/prefix_kernel.cu")  # setup.py:13-19
ARCH = "-gencode=arch=compute_103,code=sm_103"


def staged() -> bool:
    return all((PACKAGE / s).exists() for s in SOURCES) and (PACKAGE / "__init__.py").exists()


def stage(reference: Path) -> Path:
    """Copy the reference package (Python + csrc) and its tests into baseline/_ref/."""
    reference = Path(reference)
    if not (reference / "panoptic_evaluator" / "__init__.py").exists():
        raise FileNotFoundError(f"{reference} is not a panoptic-evaluator checkout")
    STAGE.mkdir(parents=True, exist_ok=True)
    for name in ("panoptic_evaluator", "tests"):
        target = STAGE / name
        if target.exists():
            shutil.rmtree(target)
        shutil.copytree(reference / name, target, ignore=shutil.ignore_patterns("__pycache__", "*.so", "*.pyc"))
    return STAGE


def build(verbose: bool = False) -> Path:
    """Compile the staged reference extension for sm_103 (skipped when it is newer than its sources)."""
    if not staged():
        raise FileNotFoundError("reference sources are not staged in baseline/_ref (run the stage step)")
    sources = [PACKAGE / s for s in SOURCES]
    if EXTENSION.exists() and all(EXTENSION.stat().st_mtime > s.stat().st_mtime for s in sources):
        return EXTENSION
    from torch.utils.cpp_extension import load
    work = STAGE / f"_build-{platform.machine()}"  # objects of one host architecture only
    work.mkdir(exist_ok=True)
    os.environ.setdefault("MAX_JOBS", str(min(8, os.cpu_count() or 1)))
    load(name="_cuda_evaluator", sources=[str(s) for s in sources], extra_cflags=["-O3"],
         extra_cuda_cflags=["-O3", ARCH], build_directory=str(work), verbose=verbose)
    built = work / "_cuda_evaluator.so"
    tmp = EXTENSION.with_suffix(".so.tmp")
    shutil.copyfile(built, tmp)
    os.replace(tmp, EXTENSION)
    return EXTENSION


def load():
    """Import the staged reference package with its own CUDA extension."""
    if not EXTENSION.exists():
        raise FileNotFoundError("the reference extension is not built (baseline/_ref)")
    import torch  # noqa: F401  (the extension links against torch's libraries)
    if str(STAGE) not in sys.path:
        sys.path.insert(0, str(STAGE))
    package = importlib.import_module("panoptic_evaluator")
    module = importlib.import_module("panoptic_evaluator._cuda_evaluator")
    if Path(getattr(module, "__file__", "")).resolve() != EXTENSION.resolve():
        raise RuntimeError(f"panoptic_evaluator._cuda_evaluator came from {getattr(module, '__file__', None)}")
    return package


def flatten(tree, prefix="", out=None):
    """Result tree (dicts / lists of tensors, arrays, scalars) -> {path: numpy array}."""
    from collections.abc import Mapping, Sequence

    import numpy as np
    out = {} if out is None else out
    if isinstance(tree, Mapping):
        for key, value in tree.items():
            flatten(value, f"{prefix}/{key}", out)
    elif isinstance(tree, Sequence) and not isinstance(tree, str):
        for i, value in enumerate(tree):
            flatten(value, f"{prefix}/{i}", out)
    else:
        out[prefix] = tree.detach().cpu().numpy() if hasattr(tree, "detach") else np.asarray(tree)
    return out


def _timed(step, warmup, steps):
    """Median over `steps` timed calls of ms per call (CUDA events on the current stream, host waits each)."""
    import statistics

    import torch
    for _ in range(warmup):
        result = step()
    torch.cuda.synchronize()
    times = []
    for _ in range(steps):
        start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        start.record()
        result = step()
        end.record()
        end.synchronize()
        times.append(start.elapsed_time(end))
    return statistics.median(times), result


def measure(plan: dict, results_path: Path) -> dict:
    """Time the reference's evaluators on CUDA over the workloads of ``plan`` (seeds and sizes).

    Every step runs through the reference's public API and its own extension,
    with inputs resident on the device: reset + update(s) + compute. The full
    results go to ``results_path`` (npz of flattened trees) for comparison.
    """
    import multiprocessing as mp

    import numpy as np

    sys.path.insert(0, str(HERE.parent))
    from functools import partial

    from panoptic_evaluator_gb300 import synthetic  # numpy only: no kernels of this library are loaded

    with mp.get_context("spawn").Pool(min(16, os.cpu_count() or 1)) as pool:  # before any CUDA call
        combined = synthetic.segmentation_batch(seed=plan["combined_seed"], images=plan["combined_images"],
                                                pool=pool) if plan.get("combined_images") else []
        instances = pool.map(partial(synthetic.instance_one, plan["instance_seed"]),
                             range(plan.get("instance_images", 0)), chunksize=1)
        prefixes = synthetic.prefix_batch(seed=plan["prefix_seed"], images=plan["prefix_images"], masks=64,
                                          pool=pool) if plan.get("prefix_images") else []
    import torch
    pe = load()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    t = lambda x: torch.from_numpy(np.ascontiguousarray(x)).to(dev)  # noqa: E731
    C, things = plan["num_classes"], plan["things"]
    isthing = [c < things for c in range(C)]
    warmup, steps = plan.get("warmup", 2), plan.get("steps", 5)
    rows, saved = {}, {}

    def record(name, images, ms, result, note):
        rows[name] = {"images": images, "ms_per_step": ms, "value": images / (ms / 1e3), "unit": "images/s",
                      "step": note}
        for key, value in flatten(result, name).items():
            saved[key] = value

    # Config 1: PanopticEvaluator, B=8 of 256 x 256, 20 classes (12 things), Voronoi maps.
    a = synthetic.voronoi_batch(seed=plan["voronoi_seed"])
    ev = pe.PanopticEvaluator(a.num_classes, isthing=a.isthing.tolist(), device=dev, validate=False)
    pred, target = pe.PanopticBatch(t(a.pred), t(a.pc)), pe.PanopticBatch(t(a.gt), t(a.gc), t(a.crowd))

    def voronoi():
        ev.reset()
        ev.update(pred, target)
        return ev.compute()
    ms, result = _timed(voronoi, warmup, steps)
    record("voronoi", a.gt.shape[0], ms, result, "PanopticEvaluator reset + update + compute")

    # Config 2: PanopticEvaluator over COCO-shape batches of 16 images on a 640 x 640 canvas.
    batches = []
    for k in range(plan.get("panoptic_batches", 0)):
        b = synthetic.coco_panoptic_batch(seed=plan["panoptic_seed"] + k)
        batches.append((pe.PanopticBatch(t(b.pred), t(b.pc)), pe.PanopticBatch(t(b.gt), t(b.gc), t(b.crowd))))
    if batches:
        pan = pe.PanopticEvaluator(C, isthing=isthing, device=dev, validate=False)

        def panoptic():
            pan.reset()
            for p, g in batches:
                pan.update(p, g)
            return pan.compute()
        ms, result = _timed(panoptic, warmup, steps)
        record("panoptic", 16 * len(batches), ms, result, "PanopticEvaluator reset + one update per batch + compute")

    # Config 3: InstanceEvaluator (COCO mask AP) over the instance batch in one update.
    if instances:
        ipred = pe.InstanceBatch([t(i.pred_masks) for i in instances], [t(i.pred_classes) for i in instances],
                                 [t(i.scores) for i in instances])
        itarget = pe.InstanceBatch([t(i.gt_masks) for i in instances], [t(i.gt_classes) for i in instances],
                                   crowd=[t(i.crowd) for i in instances])
        inst = pe.InstanceEvaluator(80, device=dev, validate=False)

        def instance():
            inst.reset()
            inst.update(ipred, itarget)
            return inst.compute()
        ms, result = _timed(instance, warmup, steps)
        record("instance", len(instances), ms, result, "InstanceEvaluator reset + update + compute")

    # Config 4: SegmentationEvaluator over uneven images; the reference takes B x H x W maps, so every
    # image of a different size is its own update (its per-image kernel path).
    if combined:
        seg = pe.SegmentationEvaluator(C, isthing=isthing, device=dev, validate=False)
        inputs = [(pe.PanopticBatch(t(i.pred[None]), t(i.pred_classes[None])),
                   pe.InstanceBatch([t(i.det_masks)], [t(i.det_classes)], [t(i.scores)]),
                   pe.PanopticBatch(t(i.target[None]), t(i.target_classes[None]), t(i.crowd[None])))
                  for i in combined]

        def segmentation():
            seg.reset()
            for p, d, g in inputs:
                seg.update(p, d, g)
            return seg.compute()
        ms, result = _timed(segmentation, 1, max(2, steps // 2))
        record("combined", len(combined), ms, result,
               "SegmentationEvaluator reset + one update per image (B = 1) + compute")

    # Generation prefixes: segmentation_prefixes over same-size images, 64 masks, checkpoints 8..64.
    if prefixes:
        ptarget = pe.PanopticBatch(t(np.stack([i.target for i in prefixes])),
                                   t(np.stack([i.target_classes for i in prefixes])),
                                   t(np.stack([i.crowd for i in prefixes])))
        ppred = pe.InstanceBatch([t(i.masks) for i in prefixes], [t(i.classes) for i in prefixes])

        def prefix():
            return pe.segmentation_prefixes(ppred, ptarget, C, isthing=isthing, checkpoints=list(range(8, 65, 8)),
                                            validate=False)
        ms, result = _timed(prefix, warmup, steps)
        record("prefix", len(prefixes), ms, result, "segmentation_prefixes, checkpoints 8..64 step 8")

    np.savez(results_path, **{k: v for k, v in saved.items()})
    mapped = Path("/proc/self/maps").read_text() if Path("/proc/self/maps").exists() else ""
    return {"rows": rows, "device": torch.cuda.get_device_name(dev),
            "extension": str(EXTENSION.relative_to(HERE.parent)), "arch": ARCH,
            "this_library_loaded": "libpe_gb300.so" in mapped}


def load_python():
    """Import the staged reference package for its CPU path (its extension is not needed or loaded)."""
    import torch  # noqa: F401
    if str(STAGE) not in sys.path:
        sys.path.insert(0, str(STAGE))
    if not (PACKAGE / "__init__.py").exists():
        raise FileNotFoundError("the reference package is not staged (baseline/_ref)")
    return importlib.import_module("panoptic_evaluator")


def measure_cpu(plan: dict, threads: int) -> dict:
    """Time the reference's own CPU evaluators (torch on the host, ``device="cpu"``, validation off).

    Bounded samples of each workload (the plan gives seeds and the number of
    images per sample): reset + update(s) + compute, median of a few rounds
    after one warm-up, as images/s, with ``torch.set_num_threads(threads)``.
    """
    import statistics
    import time

    import numpy as np
    import torch
    torch.set_num_threads(threads)
    sys.path.insert(0, str(HERE.parent))
    from panoptic_evaluator_gb300 import synthetic  # numpy only
    pe = load_python()
    t = lambda x: torch.from_numpy(np.ascontiguousarray(x))  # noqa: E731
    C, things = plan["num_classes"], plan["things"]
    isthing = [c < things for c in range(C)]
    rounds = plan.get("rounds", 3)
    rows = {}

    def timed(name, images, step, note):
        step()
        times = []
        for _ in range(rounds):
            t0 = time.perf_counter()
            step()
            times.append(time.perf_counter() - t0)
        s = statistics.median(times)
        rows[name] = {"images": images, "s_per_step": s, "value": images / s, "unit": "images/s", "step": note}

    a = synthetic.voronoi_batch(seed=plan["voronoi_seed"])
    ev = pe.PanopticEvaluator(a.num_classes, isthing=a.isthing.tolist(), device="cpu", validate=False)
    pred, target = pe.PanopticBatch(t(a.pred), t(a.pc)), pe.PanopticBatch(t(a.gt), t(a.gc), t(a.crowd))
    timed("voronoi", a.gt.shape[0], lambda: (ev.reset(), ev.update(pred, target), ev.compute()),
          "PanopticEvaluator reset + update + compute, 8 images of 256 x 256")

    b = synthetic.coco_panoptic_batch(seed=plan["panoptic_seed"])
    pan = pe.PanopticEvaluator(C, isthing=isthing, device="cpu", validate=False)
    pp, pt = pe.PanopticBatch(t(b.pred), t(b.pc)), pe.PanopticBatch(t(b.gt), t(b.gc), t(b.crowd))
    timed("panoptic", b.gt.shape[0], lambda: (pan.reset(), pan.update(pp, pt), pan.compute()),
          "PanopticEvaluator reset + update + compute, one COCO-shape batch of 16 on the 640 x 640 canvas")

    n_inst = plan.get("instance_sample", 2)
    inst_images = [synthetic.instance_one(plan["instance_seed"], i) for i in range(n_inst)]
    ip = pe.InstanceBatch([t(i.pred_masks) for i in inst_images], [t(i.pred_classes) for i in inst_images],
                          [t(i.scores) for i in inst_images])
    it = pe.InstanceBatch([t(i.gt_masks) for i in inst_images], [t(i.gt_classes) for i in inst_images],
                          crowd=[t(i.crowd) for i in inst_images])
    inst = pe.InstanceEvaluator(80, device="cpu", validate=False)
    timed("instance", n_inst, lambda: (inst.reset(), inst.update(ip, it), inst.compute()),
          f"InstanceEvaluator reset + update + compute, the first {n_inst} images of the instance batch")

    n_seg = plan.get("combined_sample", 8)
    seg_images = [synthetic.segmentation_one(plan["combined_seed"], i) for i in range(n_seg)]
    seg = pe.SegmentationEvaluator(C, isthing=isthing, device="cpu", validate=False)
    inputs = [(pe.PanopticBatch(t(i.pred[None]), t(i.pred_classes[None])),
               pe.InstanceBatch([t(i.det_masks)], [t(i.det_classes)], [t(i.scores)]),
               pe.PanopticBatch(t(i.target[None]), t(i.target_classes[None]), t(i.crowd[None]))) for i in seg_images]

    def segmentation():
        seg.reset()
        for p, d, g in inputs:
            seg.update(p, d, g)
        return seg.compute()
    timed("combined", n_seg, segmentation,
          f"SegmentationEvaluator reset + one update per image + compute, the first {n_seg} images of the "
          "256-image uneven batch")
    return {"rows": rows, "threads": threads, "torch": torch.__version__}


def main(argv=None):
    parser = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    sub = parser.add_subparsers(dest="command", required=True)
    s = sub.add_parser("stage")
    s.add_argument("--reference", required=True, type=Path, help="path of a panoptic-evaluator checkout")
    b = sub.add_parser("build")
    b.add_argument("--verbose", action="store_true")
    m = sub.add_parser("measure", help="time the reference's CUDA evaluators (prints one JSON line)")
    m.add_argument("--plan", required=True, help="JSON object of seeds and sizes")
    m.add_argument("--results", required=True, type=Path, help="npz file for the flattened results")
    mc = sub.add_parser("measure-cpu", help="time the reference's CPU evaluators (prints one JSON line)")
    mc.add_argument("--plan", required=True, help="JSON object of seeds and sample sizes")
    mc.add_argument("--threads", type=int, default=1)
    args = parser.parse_args(argv)
    if args.command == "measure":
        import json
        print(json.dumps(measure(json.loads(args.plan), args.results)), flush=True)
    elif args.command == "measure-cpu":
        import json
        print(json.dumps(measure_cpu(json.loads(args.plan), args.threads)), flush=True)
    else:
        print(stage(args.reference) if args.command == "stage" else build(args.verbose))


if __name__ == "__main__":
    main()
