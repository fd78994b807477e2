"""ctypes binding of ``libpe_gb300.so`` (declarations in ``include/pe_gb300.h``).

The library must have been built (``python -m panoptic_evaluator_gb300.build``
or ``__graft_entry__.build()``). Nothing here falls back to another
implementation: a missing library or a failing call raises.
"""

from __future__ import annotations

import contextlib
import ctypes
import os
import threading
from pathlib import Path

import torch

# PE_GB300_LIBRARY may name another build of the same ABI (for example a tuning variant).
LIBRARY = Path(os.environ.get("PE_GB300_LIBRARY", Path(__file__).resolve().parent / "libpe_gb300.so"))

P = ctypes.c_void_p
I64 = ctypes.c_int64
I32 = ctypes.c_int
D = ctypes.c_double

# name -> argument types; every entry point returns int.
SIGNATURES = {
    "pe_wait_selftest": [I64, I32, P, P],
    "pe_tune_update": [I64, I64, I32, I32, I32],
    "pe_update_choice": [I64, I64, P, P, P],
    "pe_tune_pass": [I64, I32, I32],
    "pe_pass_choice": [I64, P, P],
    "pe_update": [P, I32, P, I32, I64, I64, P, P, P, I64, I64, I64, P, P, P, P, P, P, P, P, P, P, P, P, P,
                  I32, I32, P],
    "pe_update_noalloc": [P, I32, P, I32, I64, I64, P, P, P, I64, I64, I64, P, P, P, P, P, P, P, P, P, I32, I32, P],
    "pe_compute": [P, P, P, P, P, P, I64, I64, P, P, P, P, P, P, P, P, P, P],
    "pe_pack": [P, I32, I64, I64, P, P, I64, P, P, P],
    "pe_reward_pq": [P, P, P, P, I64, I64, P, P, P, P, P, P],
    "pe_instance_histogram": [P, I64, I64, P, P, I64, P, P],
    "pe_instance_match": [P, I64, I64, P, P, P, P, P, P, I64, P, P, P, P],
    "pe_mask_overlap": [P, I64, P, I64, I64, P, P, P, P],
    "pe_instance_accumulate_workspace": [I64, I64],
    "pe_instance_accumulate": [P, P, P, I64, I64, P, I64, P, I64, P, I64, P, P, P, P],
    "pe_instance_summarize": [P, P, I64, P, P],
    "pe_desc_fields": [],
    "pe_seg_sort_workspace": [I64],
    "pe_seg_sort": [P, I64, P, P, I64, P, P, P, P, I64, P],
    "pe_seg_pass": [P, I64, I64, P, P, I64, P, I64, I64, I64, I32, P, I64, P, P, P],
    "pe_seg_score": [P, I64, I64, I64, P, P, P, P, P, P, P, P, P, P, P, P, I64, P, P, P, P, P, P, P, P, I32, I32, P, P, P],
    "pe_seg_match": [P, P, P, P, I64, P, P, P, P, P, P, I64, I64, P, I64, I64, P, P, P, P, P],
    "pe_inst_overlap": [P, I64, I64, I64, P, P, P, P, I64, P, I64, P, I64, P],
    "pe_pack_rgb": [P, I64, I64, P, P, I64, P, P, P],
    "pe_inst_contract": [P, P, I64, I64, P, I64, P, P, I64, P, I64, P, I64, P, P, P],
    "pe_contract_maps": [P, I64, P],
    "pe_contract_blocks": [P, P, P, P, I64, D, I64, P, I64, P, P, P],
    "pe_inst_gather": [P, P, I64, P, P, P, P, P, P],
    "pe_inst_prepare": [P, I64, P, P, P, P, P, P, P, P, P, I64, I32, P, P, P],
    "pe_prefix_desc_fields": [],
    "pe_prefix": [P, I64, I64, I64, I64, I64, I64, P, P, P, P, P, P, I64, I64, P, I64, P, I64, P, I64, P, I64, P, P,
                  P, P, P, P, P, P, P, P, P, P, P, P, I32, I32, P, P, P],
}

# Entry points that return a size instead of a status.
INT64_RESULTS = {"pe_instance_accumulate_workspace", "pe_seg_sort_workspace", "pe_contract_blocks"}

_lock = threading.Lock()
_lib = None


class NativeError(RuntimeError):
    """A pe_gb300 entry point reported an argument or CUDA error."""


def library():
    """Load the library once; raise if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not LIBRARY.exists():
            raise RuntimeError(
                f"{LIBRARY.name} is not built; run `python -m panoptic_evaluator_gb300.build` "
                "(this package has no CPU fallback)")
        lib = ctypes.CDLL(str(LIBRARY))
        lib.pe_last_error.restype = ctypes.c_char_p
        lib.pe_last_error.argtypes = []
        lib.pe_launch_count.restype = ctypes.c_longlong
        lib.pe_launch_count.argtypes = []
        lib.pe_reset_launch_count.restype = None
        lib.pe_reset_launch_count.argtypes = []
        lib.pe_abi_version.restype = ctypes.c_int
        for name, argtypes in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.argtypes = argtypes
            fn.restype = ctypes.c_int64 if name in INT64_RESULTS else ctypes.c_int
        _lib = lib
    if os.environ.get("PE_GB300_TUNING"):  # cached launch choices of an earlier tuning run
        from . import tuning
        tuning.load()
    return _lib


def exported_symbols():
    return ["pe_last_error", "pe_launch_count", "pe_reset_launch_count", "pe_abi_version", *SIGNATURES]


def ptr(tensor):
    """Device pointer of a tensor as an int (None for None); ctypes passes it as void*."""
    return None if tensor is None else tensor.data_ptr()


def stream_handle(device=None):
    return torch.cuda.current_stream(device).cuda_stream


def on_device(device):
    """Context making `device` current, or nothing when it already is (the common case)."""
    index = torch.device(device).index
    if index is None or index == torch.cuda.current_device():
        return contextlib.nullcontext()
    return torch.cuda.device(index)


def call(name, *args):
    """Invoke an entry point; negative statuses raise, others are returned."""
    status = getattr(library(), name)(*args)
    if status < 0:
        message = library().pe_last_error().decode(errors="replace")
        raise NativeError(f"{name}: {message} (status {status})")
    return status


def size(name, *args) -> int:
    """Invoke a size query (workspace bytes, descriptor width)."""
    return int(getattr(library(), name)(*args))


def launch_count() -> int:
    return int(library().pe_launch_count())


_SM_COUNTS: dict = {}


def sm_count(device) -> int:
    """Streaming multiprocessors of a CUDA device (cached)."""
    index = torch.device(device).index
    index = torch.cuda.current_device() if index is None else index
    if index not in _SM_COUNTS:
        _SM_COUNTS[index] = torch.cuda.get_device_properties(index).multi_processor_count
    return _SM_COUNTS[index]
