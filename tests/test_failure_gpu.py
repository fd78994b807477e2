"""Bounded device waits: a wait that never completes ends with an error status, and the context stays usable."""

import pytest
import torch

pytestmark = pytest.mark.gpu


def test_wait_that_never_completes_times_out_with_an_error_status():
    from panoptic_evaluator_gb300 import _native as N
    dev = torch.device("cuda")
    error = torch.full((1,), -1, dtype=torch.int32, device=dev)
    stream = N.stream_handle(dev)
    assert N.call("pe_wait_selftest", 2_000_000, 0, N.ptr(error), stream) == 0  # about a millisecond
    assert int(error.item()) == 1 << 30
    assert N.call("pe_wait_selftest", 2_000_000, 1, N.ptr(error), stream) == 0  # the phase completes
    assert int(error.item()) == 0
    # The context still runs work: an evaluation right after the timeout.
    import panoptic_evaluator_gb300 as pe
    maps = torch.zeros((1, 8, 8), dtype=torch.int32, device=dev)
    maps[:, 4:] = 1
    classes = torch.tensor([[-1, 0]], dtype=torch.int32, device=dev)
    pq = pe.panoptic_quality(pe.PanopticBatch(maps, classes), pe.PanopticBatch(maps, classes), num_classes=1)
    assert float(pq[0]) == 1.0


def test_wait_limit_is_checked_on_the_host():
    from panoptic_evaluator_gb300 import _native as N
    error = torch.zeros(1, dtype=torch.int32, device="cuda")
    with pytest.raises(RuntimeError):
        N.call("pe_wait_selftest", 0, 0, N.ptr(error), N.stream_handle(torch.device("cuda")))
