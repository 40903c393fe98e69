"""Tile-shape autotuning on the caller's own workload.

The kernels' tunable launch shapes are process-wide knobs of the C ABI
(``trot_set_tuning``); every setting computes bit-identical results, so tuning
only changes speed.  ``tune_exchange`` times the exact-slice exchange kernel's
work-item size (walker tiles per item) and persistent grid on one local-energy
evaluation of the given batch, keeps the fastest and caches the choice per
problem shape."""
from __future__ import annotations

import torch

from . import _lib

_cache: dict = {}

EXCHANGE_TILES = (4, 8, 16, 32, 64)
EXCHANGE_GRID = (152, 304)


def _time(fn, reps: int) -> float:
    fn()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(reps):
        fn()
    b.record()
    torch.cuda.synchronize()
    return a.elapsed_time(b) / reps


def tune_exchange(walkers, ham_data, meas_ops, meas_ctx, trial_data, reps: int = 3,
                  tiles=EXCHANGE_TILES, grids=EXCHANGE_GRID) -> dict:
    """Choose (tiles per item, grid) of the exchange kernel for this batch shape
    by timing ``meas_ops.kernels["energy"]``; sets the knobs and returns
    {"tiles": t, "grid": g, "ms": best, "timings": {...}}."""
    w0 = walkers[0] if isinstance(walkers, tuple) else walkers
    key = (tuple(w0.shape), tuple(walkers[1].shape) if isinstance(walkers, tuple) else None,
           int(getattr(meas_ctx, "rot_chol", getattr(meas_ctx, "rot_chol_a", w0)).shape[0]))
    hit = _cache.get(key)
    if hit is not None:
        set_exchange(hit["tiles"], hit["grid"])
        return hit
    energy = meas_ops.kernels["energy"]
    timings = {}
    for g in grids:
        for t in tiles:
            set_exchange(t, g)
            timings[(t, g)] = _time(lambda: energy(walkers, ham_data, meas_ctx, trial_data), reps)
    (t, g), best = min(timings.items(), key=lambda kv: kv[1])
    set_exchange(t, g)
    res = {"tiles": t, "grid": g, "ms": best, "timings": {f"{k[0]}x{k[1]}": v for k, v in timings.items()}}
    _cache[key] = res
    return res


def set_exchange(tiles: int = 0, grid: int = 0) -> None:
    """Set the exchange kernel's knobs directly (0 = built-in default)."""
    _lib.call("trot_set_tuning", _lib.TUNE_EXCHANGE_TILES, int(tiles))
    _lib.call("trot_set_tuning", _lib.TUNE_EXCHANGE_GRID, int(grid))


def reset() -> None:
    set_exchange(0, 0)
    _cache.clear()
