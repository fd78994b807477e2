"""Drop-in check: the reference's own test suite, run on its Python layer with this library as its extension.

The reference's package and tests are staged (unmodified) in the git-ignored
``baseline/_ref/`` by ``baseline/reference_cuda.py stage``. A child pytest run
loads ``tests/reference_shim.py``, which registers
``panoptic_evaluator_gb300._cuda_evaluator`` as the reference's
``panoptic_evaluator._cuda_evaluator``, then runs the reference's five test
files. Their CUDA classes and methods (``tests/test_evaluator.py:279-376``,
``test_rewards.py:103-105``, ``test_prefix.py:96-98``,
``test_instance.py:71,220,239``, ``test_combined.py:180``) drive the
reference's ``PanopticEvaluator``, ``panoptic_quality``, ``InstanceEvaluator``,
``SegmentationEvaluator`` and ``segmentation_prefixes`` on CUDA tensors through
this library's kernels and compare them with the reference's own CPU path.
"""

import os
import subprocess
import sys
import xml.etree.ElementTree as ET
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent
STAGE = ROOT / "baseline" / "_ref"
FILES = ("test_evaluator.py", "test_rewards.py", "test_prefix.py", "test_instance.py", "test_combined.py")
# Tests the reference itself skips without its optional external tools (panopticapi, pycocotools).
OPTIONAL = ("test_official_randomized_parity", "test_pycocotools")


def _is_cuda_case(case):
    name, cls = case.get("name", ""), case.get("classname", "")
    return "CUDA" in cls or "cuda" in name or name in (
        "test_nondefault_stream_snapshots_and_validation", "test_native_matcher_adversarial_parity",
        "test_nondefault_stream_and_snapshot")


def test_reference_suite_runs_on_this_library(tmp_path):
    if not all((STAGE / "tests" / f).exists() for f in FILES) or not (STAGE / "panoptic_evaluator").exists():
        pytest.skip("the reference package is not staged in baseline/_ref")
    # The library itself must be built before the child imports it.
    from panoptic_evaluator_gb300 import _native
    _native.library()
    report = tmp_path / "reference.xml"
    env = dict(os.environ)
    env["PYTHONPATH"] = os.pathsep.join([str(ROOT / "tests"), str(ROOT), str(STAGE)] +
                                        ([env["PYTHONPATH"]] if env.get("PYTHONPATH") else []))
    cmd = [sys.executable, "-m", "pytest", "-q", "-p", "reference_shim", "-p", "no:cacheprovider",
           f"--junitxml={report}", "--rootdir", str(STAGE), *[str(STAGE / "tests" / f) for f in FILES]]
    run = subprocess.run(cmd, cwd=str(tmp_path), env=env, capture_output=True, text=True, timeout=1200)
    tail = (run.stdout + run.stderr)[-4000:]
    assert run.returncode == 0, tail
    assert "reference_shim: reference layer ran on" in run.stdout, tail
    cases = ET.parse(report).getroot().iter("testcase")
    cuda_passed, cuda_skipped = [], []
    for case in cases:
        if not _is_cuda_case(case):
            continue
        skipped = case.find("skipped") is not None
        failed = case.find("failure") is not None or case.find("error") is not None
        assert not failed, case.get("name")
        if skipped:
            if not any(case.get("name", "").startswith(o) for o in OPTIONAL):
                cuda_skipped.append(case.get("classname") + "." + case.get("name"))
        else:
            cuda_passed.append(case.get("name"))
    assert not cuda_skipped, cuda_skipped
    # Every CUDA case of the reference suite ran: the evaluator, reward and prefix classes inherit their
    # CPU classes' tests, plus the CUDA methods of the instance and combined tests (28 cases, one of which
    # is the panopticapi comparison the reference skips without panopticapi).
    assert len(cuda_passed) >= 27, (len(cuda_passed), tail)
