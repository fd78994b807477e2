"""Build ``libpe_gb300.so`` (the C-ABI library of sm_103a kernels) in-tree.

Each ``csrc/*.cu`` translation unit is compiled in parallel with nvcc for
``sm_103a`` only, then linked into ``panoptic_evaluator_gb300/libpe_gb300.so``.
Objects go to ``_build/`` at the repository root. Rebuilds only when a source
or header is newer than the library.

    python -m panoptic_evaluator_gb300.build [--force] [--verbose]
"""

from __future__ import annotations

import argparse
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PACKAGE = Path(__file__).resolve().parent
CSRC = PACKAGE / "csrc"
ROOT = PACKAGE.parent
BUILD = ROOT / "_build"
LIBRARY = PACKAGE / "libpe_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC,-fvisibility=hidden",
         "-I", str(CSRC), "-I", str(ROOT / "include")]


def nvcc() -> str:
    for candidate in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if candidate and Path(candidate).exists():
            return candidate
    raise RuntimeError("nvcc not found; the CUDA toolkit is required to build libpe_gb300.so")


def sources():
    return sorted(CSRC.glob("*.cu"))


def stale() -> bool:
    if not LIBRARY.exists():
        return True
    built = LIBRARY.stat().st_mtime
    inputs = list(sources()) + list(CSRC.glob("*.cuh")) + list((ROOT / "include").glob("*.h")) + [Path(__file__)]
    return any(path.stat().st_mtime > built for path in inputs)


def build(force: bool = False, verbose: bool = False, extra: list[str] | None = None) -> Path:
    if not force and not stale():
        return LIBRARY
    compiler = nvcc()
    BUILD.mkdir(exist_ok=True)
    extra = list(extra or [])

    def compile_one(src: Path) -> Path:
        obj = BUILD / (src.stem + ".o")
        cmd = [compiler, *ARCH, *FLAGS, *extra, "-c", str(src), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd), flush=True)
        result = subprocess.run(cmd, capture_output=True, text=True)
        if result.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src.name}:\n{result.stdout}\n{result.stderr}")
        if verbose and (result.stdout or result.stderr):
            print(result.stdout + result.stderr, flush=True)
        return obj

    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as pool:
        objects = list(pool.map(compile_one, sources()))
    tmp = LIBRARY.with_suffix(".so.tmp")
    cmd = [compiler, *ARCH, "-shared", "-o", str(tmp), *map(str, objects), "-lcudart"]
    result = subprocess.run(cmd, capture_output=True, text=True)
    if result.returncode != 0:
        raise RuntimeError(f"link failed:\n{result.stdout}\n{result.stderr}")
    os.replace(tmp, LIBRARY)
    return LIBRARY


def main(argv=None):
    parser = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    parser.add_argument("--force", action="store_true")
    parser.add_argument("--verbose", action="store_true")
    parser.add_argument("--ptxas-info", action="store_true", help="print registers/spills per kernel")
    args = parser.parse_args(argv)
    extra = ["-Xptxas", "-v"] if args.ptxas_info else None
    path = build(force=args.force or args.ptxas_info, verbose=args.verbose or args.ptxas_info, extra=extra)
    print(path)


if __name__ == "__main__":
    sys.exit(main())
