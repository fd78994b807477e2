"""The C-ABI library loads here (no GPU needed) and exports every declared entry point."""

import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def declared_symbols():
    text = (ROOT / "include" / "pe_gb300.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(pe_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "pe_update" in names and "pe_compute" in names and "pe_pack" in names


def test_library_exports_every_declared_symbol():
    from panoptic_evaluator_gb300 import build, _native
    build.build()
    lib = _native.library()
    for name in declared_symbols():
        assert hasattr(lib, name), name
    assert set(declared_symbols()) == set(_native.exported_symbols())
    assert lib.pe_abi_version() >= 1


def test_product_fails_loudly_without_cuda_tensors():
    import torch
    from panoptic_evaluator_gb300 import PanopticBatch, PanopticEvaluator
    with pytest.raises(ValueError):
        PanopticEvaluator(3, device="cpu")
    if not torch.cuda.is_available():
        with pytest.raises((ValueError, RuntimeError)):
            PanopticEvaluator(3)
