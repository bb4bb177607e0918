"""Launch-shape autotuner.

Times every kernel shape the library offers on a sample of the caller's
workload, keeps the fastest, and caches the choice per GPU name in
``ochre_gb300/_build/tune.json``:
  * the fused small-raster kernel: threads per raster and tiles per
    accumulation pass;
  * tiles per warp of the general chain's coverage kernel;
  * the digit width of the chain's radix sort (8 or 11 bits).
Results never depend on the shape (tile and span structure is exact, alpha
within 1 LSB of the oracle either way; the sort is stable at any width).
"""
from __future__ import annotations

import ctypes
import json
import os
import time
from typing import Optional

from . import _lib, build

FUSED_SHAPES = [(64, 8), (64, 16), (64, 32), (96, 8), (96, 16), (128, 16), (128, 32)]


def fused_candidates() -> list:
    """Every fused shape as the tunables that select it."""
    return [{"fused_threads": t, "fused_chunk": c} for t, c in FUSED_SHAPES]


def shape_name(p: dict) -> str:
    return f"{p['fused_threads']}x{p['fused_chunk']}"
CHAIN_TILES_PER_WARP = [4, 8, 16]
SORT_DIGIT_BITS = [8, 11]
CACHE = os.path.join(build.BUILD, "tune.json")


def gpu_name(device: int = 0) -> str:
    import torch
    return torch.cuda.get_device_name(device)


def load_cache() -> dict:
    if os.path.exists(CACHE):
        try:
            with open(CACHE) as f:
                return json.load(f)
        except (OSError, ValueError):
            return {}
    return {}


def cached(device: int = 0) -> Optional[dict]:
    return load_cache().get(gpu_name(device))


def apply(ctx, params: dict) -> None:
    L = _lib.load()
    for k, v in params.items():
        _lib.check(L.ochre_gpu_set_tunable(ctx.handle, k.encode(), int(v)), f"set_tunable {k}")


def get(ctx, name: str) -> int:
    v = ctypes.c_int()
    _lib.check(_lib.load().ochre_gpu_get_tunable(ctx.handle, name.encode(), ctypes.byref(v)))
    return v.value


def _time(ctx, dbatch, reps: int) -> float:
    import torch
    stream = torch.cuda.current_stream()
    ctx.rasterize_device(dbatch, stream.cuda_stream)
    torch.cuda.synchronize()
    best = float("inf")
    for _ in range(reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        ctx.rasterize_device(dbatch, stream.cuda_stream)
        b.record(stream)
        torch.cuda.synchronize()
        best = min(best, a.elapsed_time(b))
    return best


def tune(ctx, fused_sample=None, chain_sample=None, reps: int = 3, save: bool = True) -> dict:
    """Pick the fastest shapes on the given samples (Batch objects), apply
    them to ``ctx`` and cache them for this GPU.  Returns the choice and the
    measured times."""
    from .rasterizer import DeviceBatch
    from . import workloads as W
    fused_sample = fused_sample if fused_sample is not None else W.glyph_run(n_paths=20_000, seed=99)
    # the chain's heavy case: paths too large for the fused kernel, many tile rows
    # (4,000 paths: on 1,000 the tiles-per-warp ranking flips from run to run)
    chain_sample = chain_sample if chain_sample is not None else W.uneven_mix(n_paths=4000, seed=99)
    t0 = time.time()
    report = {"fused": {}, "chain": {}}
    old_chain = ctx.chain_only
    db = DeviceBatch(fused_sample, ctx.device)
    ctx.set_chain_only(False)
    best_f, best_t = None, float("inf")
    for cand in fused_candidates():
        apply(ctx, cand)
        ms = _time(ctx, db, reps)
        report["fused"][shape_name(cand)] = ms
        if ctx.stats().get("fused") and ms < best_t:
            best_f, best_t = cand, ms
    db = DeviceBatch(chain_sample, ctx.device)
    ctx.set_chain_only(True)
    best_c, best_ct = None, float("inf")
    for tpw in CHAIN_TILES_PER_WARP:
        apply(ctx, {"chain_tiles_per_warp": tpw})
        ms = _time(ctx, db, reps)
        report["chain"][str(tpw)] = ms
        if ms < best_ct:
            best_c, best_ct = tpw, ms
    apply(ctx, {"chain_tiles_per_warp": best_c or 8})
    # radix sort digit width on the same sample (its keys span about 30 bits:
    # four 8-bit passes or three of at most 11)
    report["sort_digit_bits"] = {}
    best_d, best_dt = None, float("inf")
    for bits in SORT_DIGIT_BITS:
        apply(ctx, {"sort_digit_bits": bits})
        ms = _time(ctx, db, reps)
        report["sort_digit_bits"][str(bits)] = ms
        if ms < best_dt:
            best_d, best_dt = bits, ms
    ctx.set_chain_only(old_chain)
    choice = dict(best_f or {"fused_threads": 64, "fused_chunk": 16})
    choice["chain_tiles_per_warp"] = best_c or 8
    choice["sort_digit_bits"] = best_d or 8
    apply(ctx, choice)
    if save:
        cache = load_cache()
        cache[gpu_name(ctx.device)] = choice
        os.makedirs(build.BUILD, exist_ok=True)
        with open(CACHE, "w") as f:
            json.dump(cache, f, indent=1)
    return {"choice": choice, "ms": report, "tune_s": time.time() - t0}
