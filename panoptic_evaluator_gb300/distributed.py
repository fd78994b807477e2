"""Replica evaluation across processes (one GPU each): merge evaluator state, then compute anywhere.

Images are independent, so N processes evaluate disjoint shares of the data
with their own evaluator and exchange state only before ``compute``:

* integer counters (tp / fp / fn / confusion / instance positives) are summed;
* FP64 sums (``iou_sum``) are summed in rank order, so every rank gets the
  same bits whatever the arrival order;
* instance records (score, class, rank, 40 match flags per detection) are
  concatenated in rank order. With a contiguous split of the images
  (rank 0 the first share, rank 1 the next, ...) the merged records are in
  the same order as one evaluator that saw every image, so ties in the global
  score sort resolve identically.

``merge_states`` does this on the host for a list of state dicts (replicas in
one process); ``all_reduce_states`` does it over a ``torch.distributed``
process group (NCCL for CUDA state, gloo for CPU state); ``sync`` replaces an
evaluator's state with the merged state of the whole group.
"""

from __future__ import annotations

from typing import Sequence

import torch
import torch.distributed as dist

RECORDS = "records."


def _kind(key: str, value: torch.Tensor) -> str:
    name = key.rsplit("/", 1)[-1]
    if name.startswith(RECORDS):
        return "concat"
    return "ordered_sum" if value.is_floating_point() else "sum"


def merge_states(states: Sequence[dict]) -> dict:
    """Merged state of several replicas, in the given (rank) order."""
    if not states:
        raise ValueError("no states to merge")
    keys = list(states[0])
    for state in states[1:]:
        if list(state) != keys:
            raise ValueError("replica states have different keys")
    merged = {}
    for key in keys:
        values = [state[key] for state in states]
        kind = _kind(key, values[0])
        if kind == "concat":
            merged[key] = torch.cat(values)
        else:
            total = values[0].clone()
            for value in values[1:]:  # fixed order: deterministic FP64 sums
                total += value
            merged[key] = total
    return merged


def _gather(tensor: torch.Tensor, group, world: int) -> list:
    """all_gather of tensors whose first dimension may differ between ranks."""
    length = torch.tensor([tensor.shape[0]], dtype=torch.int64, device=tensor.device)
    lengths = [torch.zeros_like(length) for _ in range(world)]
    dist.all_gather(lengths, length, group=group)
    lengths = [int(n.item()) for n in lengths]
    longest = max(lengths)
    padded = tensor.new_zeros((longest,) + tuple(tensor.shape[1:]))
    padded[: tensor.shape[0]] = tensor
    parts = [torch.empty_like(padded) for _ in range(world)]
    dist.all_gather(parts, padded, group=group)
    return [part[:n] for part, n in zip(parts, lengths)]


def all_reduce_states(state: dict, group=None) -> dict:
    """Merged state of every rank of `group` (the same on all ranks)."""
    world = dist.get_world_size(group)
    merged = {}
    for key, value in state.items():
        kind = _kind(key, value)
        if kind == "sum":
            total = value.clone()
            dist.all_reduce(total, op=dist.ReduceOp.SUM, group=group)
            merged[key] = total
            continue
        parts = _gather(value.contiguous() if value.dim() else value.reshape(1), group, world)
        if kind == "concat":
            merged[key] = torch.cat(parts)
        else:
            total = parts[0].clone()
            for part in parts[1:]:
                total += part
            merged[key] = total.reshape(value.shape)
    return merged


def sync(evaluator, group=None):
    """Replace `evaluator`'s state with the merged state of the group; returns the evaluator."""
    evaluator.load_state_dict(all_reduce_states(evaluator.state_dict(), group))
    return evaluator
