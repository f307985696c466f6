"""Autotuner for the occlusion kernel's launch shape.

Knobs (vxl_tuning): ray-tile shape (tile_px pixels per warp tile, laid out as
runs of pixels or 8- / 4-wide image blocks), KSTEP (DDA iterations between
pool refills), queue granularity (tiles per work-queue access) and dispatch
order. The brick size is fixed by the data layout: one 4x4x4 brick is one
64-bit word, the largest unit a thread keeps in registers, so it is not a
tuning knob.

The search is a coordinate descent from the current setting (each knob in
turn, keeping the best), timing `steps` runs of a caller-supplied step with
CUDA events. Results are cached per device name and workload key in
tuning_cache.json next to this file; `apply_cached` installs a cached entry.
"""
from __future__ import annotations

import json
import os

HERE = os.path.dirname(os.path.abspath(__file__))
CACHE = os.path.join(HERE, "tuning_cache.json")

SHAPES = [(16, 16), (16, 8), (16, 4), (32, 32), (32, 8)]  # (tile_px, tile_w)
KSTEPS = [2, 4, 8, 16]
GRABS = [1, 2, 4]
ORDERS = [1, 2]


def device_key() -> str:
    import torch

    return torch.cuda.get_device_name(0)


def load_cache() -> dict:
    if os.path.exists(CACHE):
        with open(CACHE) as f:
            return json.load(f)
    return {}


def apply_cached(ctx, workload: str) -> dict | None:
    """Install the cached tuning for (this device, workload); returns it or None."""
    entry = load_cache().get(device_key(), {}).get(workload)
    if entry:
        t = entry["tuning"]
        ctx.set_tuning(tile_px=t["tile_px"], kstep=t["kstep"], leap=t["leap"], order=t["order"], tile_w=t["tile_w"],
                       grab=t["grab"])
    return entry


def _time(make_step, steps: int, warmup: int) -> float:
    import torch

    step = make_step()
    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(steps):
        step()
    b.record()
    torch.cuda.synchronize()
    return a.elapsed_time(b) / steps


def tune(ctx, make_step, workload: str, steps: int = 10, warmup: int = 3, save: bool = True, log=None) -> dict:
    """Coordinate search. make_step() builds a zero-argument callable that
    runs one step with the context's current tuning (rebuild batches inside,
    since a batch captures the tuning when it is created)."""
    cur = ctx.get_tuning()
    best_ms = _time(make_step, steps, warmup)
    trials = [(dict(cur), best_ms)]

    def trial(**kw):
        nonlocal cur, best_ms
        cand = dict(cur)
        cand.update(kw)
        ctx.set_tuning(**cand)
        got = ctx.get_tuning()
        ms = _time(make_step, steps, warmup)
        trials.append((got, ms))
        if log:
            log("tune %s: %.3f ms" % (got, ms))
        if ms < best_ms:
            best_ms, cur = ms, got
        ctx.set_tuning(**cur)

    for tp, tw in SHAPES:
        trial(tile_px=tp, tile_w=tw)
    for k in KSTEPS:
        trial(kstep=k)
    for g in GRABS:
        trial(grab=g)
    for o in ORDERS:
        trial(order=o)
    ctx.set_tuning(**cur)
    entry = {"tuning": cur, "ms": best_ms, "trials": [{"tuning": t, "ms": m} for t, m in trials]}
    if save:
        cache = load_cache()
        cache.setdefault(device_key(), {})[workload] = entry
        with open(CACHE, "w") as f:
            json.dump(cache, f, indent=1, sort_keys=True)
    return entry
