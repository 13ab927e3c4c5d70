"""Autotuner of the launch shapes of the stacking path (sst_tuning).

The shapes it chooses among are the ones the kernels offer at run time:

  pass_ctas_per_sm      CTAs per SM of the persistent Gauss-Newton passes
  pass_tile_w[class]    64- or 128-wide tiles of the staged IC / IC-LM pass,
                        per level-width class (<= 192, <= 384, <= 768, wider)
  corr_ctas_per_sm      CTAs per SM of the correlation
  stack_max_chunks,     how far the stack splits a tile's frames over CTAs
  stack_items_per_slot

Each candidate is timed with CUDA events on the caller's stream around a full
sst_stack_frames call (registration + warp + stack) on a sample of the
caller's own device-resident frames: one untimed run, then the median of
`reps` timed runs. The search is coordinate descent in the order above,
starting from the defaults. The choice is cached on disk (JSON), keyed by the
device name and the workload's geometry (frame size, depth, pyramid levels,
method, motion passes, weighting and the power of two of the frames per
call), so a later run with the same key applies it without searching.

Cache file: $SST_TUNE_CACHE, else serstacker_gb300/_tune/tuning.json.
"""
from __future__ import annotations

import json
import os
import time
from typing import Optional, Sequence

from . import capi as C

_HERE = os.path.dirname(os.path.abspath(__file__))


def cache_path() -> str:
    return os.environ.get("SST_TUNE_CACHE") or os.path.join(_HERE, "_tune", "tuning.json")


def _load() -> dict:
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(db: dict):
    p = cache_path()
    os.makedirs(os.path.dirname(p), exist_ok=True)
    tmp = p + ".tmp"
    with open(tmp, "w") as f:
        json.dump(db, f, indent=1, sort_keys=True)
    os.replace(tmp, p)


def workload_key(device_name: str, width: int, height: int, depth: int, levels: int, method: int,
                 passes: Sequence[int], weighting: int, n: int) -> str:
    nb = 1
    while nb < n:
        nb *= 2
    return (f"{device_name}|{width}x{height}|depth{depth}|L{levels}|m{method}|"
            f"p{'-'.join(str(p) for p in passes)}|w{weighting}|n{nb}")


def _width_classes(reg: C.c_ecch) -> list:
    cls = set()
    for l in range(reg.num_levels()):
        w = reg.level_shape(l)[1]
        cls.add(0 if w <= 192 else 1 if w <= 384 else 2 if w <= 768 else 3)
    return sorted(cls)


def tune_stack_frames(reg: C.c_ecch, acc: C.c_weigthed_average, frames, n: int, width: int, height: int, depth: int,
                      row_stride: int, frame_stride: int, passes: Sequence[int], scale: float, weighting: int = 1,
                      sample: int = 512, reps: int = 3, use_cache: bool = True, method: Optional[int] = None) -> dict:
    """Choose and apply the launch shapes for sst_stack_frames on device frames.

    frames: a CUDA tensor (or device pointer) of n frames; the first
    min(n, sample) are timed. Returns {"tuning": ..., "source": "cache" |
    "search", "ms": per-call time of the chosen shapes on the sample,
    "default_ms": the defaults' time, "candidates": number timed, "key": ...}.
    """
    import torch
    dev = torch.cuda.current_device()
    name = torch.cuda.get_device_name(dev)
    method = reg.options.method if method is None else method
    key = workload_key(name, width, height, depth, reg.num_levels(), method, passes, weighting, n)
    db = _load() if use_cache else {}
    if key in db:
        t = db[key]["tuning"]
        reg.set_tuning(t)
        acc.set_tuning(t)
        return {"tuning": t, "source": "cache", "ms": db[key].get("ms"), "default_ms": db[key].get("default_ms"),
                "candidates": db[key].get("candidates"), "key": key}

    ns = max(1, min(n, sample))
    outs = {"params": torch.zeros((ns, 12), dtype=torch.float32, device="cuda"),
            "status": torch.zeros(ns, dtype=torch.int32, device="cuda"),
            "rho": torch.zeros(ns, dtype=torch.float32, device="cuda"),
            "weight": torch.zeros(ns, dtype=torch.float32, device="cuda")}
    ptr = frames.data_ptr() if hasattr(frames, "data_ptr") else int(frames)
    counted = [0]

    def run(t: dict) -> float:
        reg.set_tuning(t)
        acc.set_tuning(t)
        reg.set_chunk_frames(ns)

        def once():
            acc.clear()
            C.stack_frames(reg, acc, ptr, passes, scale, weighting=weighting, on_device=True, n=ns, width=width,
                           height=height, depth=depth, row_stride=row_stride, frame_stride=frame_stride,
                           outputs=outs)
        once()
        torch.cuda.synchronize()
        ts = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            once()
            e1.record()
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
        counted[0] += 1
        ts.sort()
        return ts[len(ts) // 2]

    t0 = time.perf_counter()
    best = {"pass_ctas_per_sm": 0, "pass_tile_w": [0, 0, 0, 0], "corr_ctas_per_sm": 0, "stack_max_chunks": 0,
            "stack_items_per_slot": 0}
    best_ms = default_ms = run(best)

    def try_field(field, values, index=None):
        nonlocal best, best_ms
        for v in values:
            cand = json.loads(json.dumps(best))
            if index is None:
                if cand[field] == v:
                    continue
                cand[field] = v
            else:
                if cand[field][index] == v:
                    continue
                cand[field][index] = v
            ms = run(cand)
            if ms < best_ms * 0.995:
                best, best_ms = cand, ms

    try_field("pass_ctas_per_sm", [1, 2, 3, 4, 6])
    if method in (C.IC, C.ICLM):
        for c in _width_classes(reg):
            try_field("pass_tile_w", [64, 128], index=c)
    try_field("corr_ctas_per_sm", [2, 8])
    try_field("stack_max_chunks", [1, 2, 8])
    try_field("stack_items_per_slot", [2, 8])
    reg.set_tuning(best)
    acc.set_tuning(best)
    entry = {"tuning": best, "ms": best_ms, "default_ms": default_ms, "candidates": counted[0], "sample": ns,
             "search_s": time.perf_counter() - t0, "device": name}
    if use_cache:
        db = _load()
        db[key] = entry
        _store(db)
    return {"tuning": best, "source": "search", "ms": best_ms, "default_ms": default_ms, "candidates": counted[0],
            "search_s": entry["search_s"], "key": key}
