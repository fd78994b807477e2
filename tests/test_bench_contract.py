"""bench.py's JSON line for the reference arm (the CPU restatement timed on the host cores): no GPU needed."""

import json
import os
import subprocess
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent


def test_reference_arm_prints_one_contract_line():
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    run = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "1", "--images", "3"], cwd=ROOT, env=env, capture_output=True, text=True,
                         timeout=600)
    assert run.returncode == 0, run.stderr[-2000:]
    lines = [line for line in run.stdout.splitlines() if line.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    for key in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference" and line["n_gpus"] == 1 and line["steps"] == 1 and line["warmup"] == 1
    assert line["higher_is_better"] is True and line["value"] > 0 and line["unit"] == "images/s"
    assert line["config"]["images"] == 3
    cpu = line["cpu_baseline"]
    assert cpu["kind"] in ("port", "reference") and cpu["cores"] >= 1 and cpu["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"], "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}


def test_grid_workload_shapes():
    """The workload of the reference's recorded timings: grid cells, void prediction rows, dilated things."""
    from panoptic_evaluator_gb300 import synthetic
    images, things = synthetic.grid_batch(seed=1, images=2, height=40, width=60, segments=16, detections=9,
                                          num_classes=15)
    assert things == [c < 10 for c in range(15)]
    for im in images:
        assert im.target.shape == (40, 60) and set(np.unique(im.target)) == set(range(1, 17))
        assert (im.target[:10, :15] == 1).all() and (im.target[10:20, 15:30] == 6).all()  # 10 x 15 cells
        assert (im.pred[:3] == 0).all() and (im.pred[3:] == im.target[3:]).all()
        assert im.target_classes[0] == -1 and im.target_classes[1] == 0 and not im.crowd[0]
        assert im.det_masks.shape == (9, 40, 60) and len(im.det_classes) == len(im.scores) == 9
        for mask, cls in zip(im.det_masks, im.det_classes):
            slot = np.bincount(im.target[mask], minlength=17).argmax()
            assert things[cls] and im.target_classes[slot] == cls
            inside = im.target == slot
            assert mask[inside].all() and mask.sum() > inside.sum()  # the dilation reaches the neighbours


def test_parity_check_of_the_bench_sections():
    """The bench's result-against-oracle check: integers exact, FP64 within 1e-12, NaN where the oracle has NaN."""
    sys.path.insert(0, str(ROOT))
    import bench
    expected = {"tp": np.array([3, 0, 2]), "All": {"pq": np.float64(0.25), "n": np.int64(2)},
                "per_class": {"iou": np.array([0.5, np.nan])}, "rows": [np.array([1.0]), np.array([2.0])]}
    same = {"tp": np.array([3, 0, 2]), "All": {"pq": 0.25 + 4e-13, "n": 2},
            "per_class": {"iou": np.array([0.5, np.nan])}, "rows": [np.array([1.0]), np.array([2.0])], "extra": 1}
    parity = bench.Parity().compare(same, expected)
    assert parity.ok() and parity.int_exact and 0 < parity.max_abs <= bench.PARITY_TOL
    assert parity.summary("oracle")["leaves"] == 6
    for broken in ({**same, "tp": np.array([3, 1, 2])}, {**same, "All": {"pq": 0.25 + 1e-9, "n": 2}},
                   {**same, "per_class": {"iou": np.array([0.5, 0.0])}}, {**same, "rows": [np.array([1.0])]},
                   {k: v for k, v in same.items() if k != "tp"}):
        parity = bench.Parity().compare(broken, expected)
        assert not parity.ok()
        try:
            parity.require("section")
        except RuntimeError as exc:
            assert "section" in str(exc)
        else:
            raise AssertionError("a mismatch must raise")
    assert not bench.Parity().compare({**same, "tp": np.array([3, 1, 2])}, expected).int_exact


def test_images_beyond_32_bit_bins_are_rejected():
    from panoptic_evaluator_gb300._batch import MAX_IMAGE_PIXELS, check_pixels
    check_pixels(np.array([1, MAX_IMAGE_PIXELS]))
    check_pixels(np.zeros(0, np.int64))
    try:
        check_pixels(np.array([5, MAX_IMAGE_PIXELS + 1]))
    except ValueError as exc:
        assert "32-bit" in str(exc)
    else:
        raise AssertionError("an image of 2^32 pixels must be rejected")
