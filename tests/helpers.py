"""Shared comparison helpers for the GPU parity tests."""

from __future__ import annotations

from collections.abc import Mapping, Sequence

import numpy as np
import torch

RTOL = ATOL = 1e-12  # FP64 tolerance; integers are compared exactly


def cuda(x, dtype=None):
    t = torch.as_tensor(np.asarray(x))
    if dtype is not None:
        t = t.to(dtype)
    return t.cuda()


def to_numpy(value):
    if isinstance(value, torch.Tensor):
        return value.detach().cpu().numpy()
    return np.asarray(value)


def assert_tree(actual, expected, path="result", exact_float=False):
    """Compare nested dict/list results: ints exactly, floats within 1e-12."""
    if isinstance(expected, Mapping):
        missing = set(expected) - set(actual)
        assert not missing, (path, missing)
        for key in expected:
            assert_tree(actual[key], expected[key], f"{path}/{key}", exact_float)
    elif isinstance(expected, Sequence) and not isinstance(expected, str):
        assert len(actual) == len(expected), path
        for i, (a, e) in enumerate(zip(actual, expected)):
            assert_tree(a, e, f"{path}/{i}", exact_float)
    else:
        a, e = to_numpy(actual), to_numpy(expected)
        assert a.shape == e.shape, (path, a.shape, e.shape)
        if e.dtype.kind in "iub":
            np.testing.assert_array_equal(a, e, err_msg=path)
        else:
            tol = 0 if exact_float else ATOL
            np.testing.assert_allclose(a, e, rtol=0 if exact_float else RTOL, atol=tol, equal_nan=True,
                                       err_msg=path)
