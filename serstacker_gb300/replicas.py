"""Replicas: one process per GPU, each stacking a contiguous range of frames.

Frames are independent once the reference pyramid is built, so a sequence
shards by frame ranges with no exchange on the data path. The only
collective is at the end: every rank saves its compensated accumulator
state, the states are gathered over the process group (gloo on the host),
and they are merged in rank order with the library's TwoSum merge
(``sst_state_merge``), so every run gives the same planes. A rank that
fails or never joins makes the gather on the other ranks end with an error
within the process group's timeout; partial results are never merged.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import capi


def frame_range(n: int, world: int, rank: int):
    """Contiguous share [lo, hi) of n frames for `rank` of `world`: the first
    n % world ranks take one frame more."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("invalid world / rank")
    q, r = divmod(n, world)
    lo = rank * q + min(rank, r)
    return lo, lo + q + (1 if rank < r else 0)


def merge_states(states) -> np.ndarray:
    """Merge accumulator states (each (G, 4, h, w) or (4, h, w) f32) in list order."""
    first = np.ascontiguousarray(states[0], np.float32)
    groups = 1 if first.ndim == 3 else first.shape[0]
    plane = first.shape[-1] * first.shape[-2]
    out = first.copy()
    for s in states[1:]:
        src = np.ascontiguousarray(s, np.float32)
        if src.shape != first.shape:
            raise ValueError("states of different shapes")
        rc = capi.lib().sst_state_merge(out.ctypes.data, src.ctypes.data, groups, C.c_size_t(plane))
        if rc != 0:
            raise capi.SSTError(f"sst_state_merge: {capi.last_error()}")
    return out


def gather_and_merge(state: np.ndarray, frames: int, group=None):
    """All ranks: gather every rank's (state, frames) over `group` (an
    initialised torch.distributed process group, gloo) and merge them in rank
    order. Returns (merged state, total frames) on every rank."""
    import torch
    import torch.distributed as dist
    world = dist.get_world_size(group)
    local = torch.from_numpy(np.ascontiguousarray(state, np.float32))
    parts = [torch.empty_like(local) for _ in range(world)]
    dist.all_gather(parts, local, group=group)
    counts = [torch.zeros(1, dtype=torch.int64) for _ in range(world)]
    dist.all_gather(counts, torch.tensor([frames], dtype=torch.int64), group=group)
    merged = merge_states([p.numpy() for p in parts])
    return merged, int(sum(int(c.item()) for c in counts))
