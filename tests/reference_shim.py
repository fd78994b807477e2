"""pytest plugin: the reference's own Python layer driving this library through the extension shim.

Loaded with ``-p reference_shim`` in a child pytest run over the reference's
test files (``test_reference_dropin_gpu.py``). Before the reference package is
imported it registers ``panoptic_evaluator_gb300._cuda_evaluator`` as
``panoptic_evaluator._cuda_evaluator``, the module the reference imports at
``evaluator.py:9-12`` (and ``instance.py``, ``combined.py``, ``prefix.py``), so
every CUDA op of the reference's evaluators runs this library's kernels. That
is the import swap a maintainer makes to adopt the library.

PIL is imported by the reference's ``tests/test_evaluator.py`` only to write
PNGs for the panopticapi comparison, which is skipped without panopticapi; a
stand-in module lets the file import where PIL is absent.

At the end of the session the plugin fails the run if any reference-built
``_cuda_evaluator`` binary was mapped into the process, and if the library's
own ``libpe_gb300.so`` was not.
"""

from __future__ import annotations

import sys
import types
from pathlib import Path

import pytest

import panoptic_evaluator_gb300._cuda_evaluator as shim

sys.modules["panoptic_evaluator._cuda_evaluator"] = shim
try:
    import PIL  # noqa: F401
except ImportError:
    stand_in = types.ModuleType("PIL")
    stand_in.Image = None
    sys.modules["PIL"] = stand_in


def _mapped_files():
    maps = Path("/proc/self/maps")
    if not maps.exists():
        return set()
    return {line.split()[-1] for line in maps.read_text().splitlines() if line.count("/")}


@pytest.hookimpl(trylast=True)
def pytest_sessionfinish(session, exitstatus):
    evaluator = sys.modules.get("panoptic_evaluator.evaluator")
    in_use = getattr(evaluator, "_cuda_evaluator", None)
    files = _mapped_files()
    foreign = sorted(f for f in files if "_cuda_evaluator" in Path(f).name and f.endswith(".so"))
    ours = sorted(f for f in files if Path(f).name == "libpe_gb300.so")
    if in_use is not shim or foreign or (files and not ours):
        print(f"reference_shim: extension in use {in_use!r}, foreign binaries "
              f"{foreign}, library {ours}", flush=True)
        session.exitstatus = pytest.ExitCode.TESTS_FAILED
    else:
        print(f"reference_shim: reference layer ran on {ours[0] if ours else 'libpe_gb300.so'}", flush=True)
