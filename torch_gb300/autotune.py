"""Tile-shape autotuner for the batched step.

For a set of grids, time a few steps of every candidate tile configuration
(in-plane tile shape, marching chunk, one CTA per tile or a persistent grid)
on scratch copies of the grids, and return the fastest.  Results are cached
per GPU, dimension, precision and grid-size signature in
``$TORCH_GB300_CACHE`` (default ``~/.cache/torch_gb300/autotune.json``).
"""

import copy
import hashlib
import json
import os
from pathlib import Path

import torch

from .batch import Batch

CACHE = Path(os.environ.get("TORCH_GB300_CACHE",
                            Path.home() / ".cache" / "torch_gb300" / "autotune.json"))


def candidates(dim, precision, sms):
    """Tile configurations (tx, ty, chunk, persistent_ctas, tma) worth trying."""
    out = []
    if dim == 3:
        shapes = [(16, 16), (32, 8)] if precision == "fp32" else [(32, 4), (16, 8)]
        for tx, ty in shapes:
            for chunk in (16, 32, 40, 64):
                out.append((tx, ty, chunk, 0, 1))
    elif dim == 2:
        # 124: rows of 124 cells whose two ring cells take the lanes after the
        # owners (single precision only: double precision tiles are whole warps)
        for tx in ((124, 128, 256) if precision == "fp32" else (128, 256)):
            for chunk in (16, 32, 64):
                for pers in (0, 2 * sms):
                    out.append((tx, 1, chunk, pers, 1))
    else:
        for tx in (128, 256):
            for pers in (0, 2 * sms):
                out.append((tx, 1, 1, pers, 0))
    return out


def signature(grids):
    g0 = grids[0]
    sizes = sorted(tuple(g.counts) for g in grids)
    key = json.dumps([torch.cuda.get_device_name(g0.device), g0.dim, g0.precision,
                      sizes, [bool(g.reactive) for g in grids]])
    return hashlib.sha1(key.encode()).hexdigest()


def _load_cache():
    try:
        return json.loads(CACHE.read_text())
    except (OSError, ValueError):
        return {}


def _store_cache(data):
    try:
        CACHE.parent.mkdir(parents=True, exist_ok=True)
        CACHE.write_text(json.dumps(data, indent=1))
    except OSError:
        pass


def _scratch_copy(grid):
    g = copy.copy(grid)
    g.ring = [t.clone() for t in grid.ring]
    g.lam_ring = None if grid.lam_ring is None else [t.clone() for t in grid.lam_ring]
    g.beta_ring = None if grid.beta_ring is None else [t.clone() for t in grid.beta_ring]
    g.report = None if grid.report is None else copy.copy(grid.report)
    return g


def time_config(grids, tile, steps=4, warmup=2):
    """Milliseconds per batched step of `tile` on scratch copies of `grids`."""
    scratch = [_scratch_copy(g) for g in grids]
    b = Batch(scratch, tile=tile)
    try:
        b.advance(warmup)
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record(b.stream)
        b.advance(steps)
        e.record(b.stream)
        e.synchronize()
        return s.elapsed_time(e) / steps
    finally:
        b.close()


def tune(grids, steps=4, warmup=2, use_cache=True, verbose=False):
    """Best tile configuration for advancing `grids` together."""
    key = signature(grids)
    cache = _load_cache() if use_cache else {}
    if key in cache:
        return tuple(cache[key]["tile"])
    sms = torch.cuda.get_device_properties(grids[0].device).multi_processor_count
    best, best_ms, results = None, float("inf"), []
    for tile in candidates(grids[0].dim, grids[0].precision, sms):
        try:
            ms = time_config(grids, tile, steps, warmup)
        except (RuntimeError, ValueError):
            continue
        results.append((tile, ms))
        if verbose:
            print("autotune", tile, f"{ms:.3f} ms")
        if ms < best_ms:
            best, best_ms = tile, ms
    if best is None:
        raise RuntimeError("no tile configuration ran")
    if use_cache:
        cache = _load_cache()
        cache[key] = {"tile": list(best), "ms": best_ms,
                      "tried": [[list(t), m] for t, m in results]}
        _store_cache(cache)
    return best
