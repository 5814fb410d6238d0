"""Pattern-tile autotuner for the mixed-precision traversal kernel.

The traversal kernel's CTA holds ``tile`` patterns x ncat threads. The best
tile depends on the state count (registers per thread), the category count
and the number of patterns (how many CTAs fill the 152 SMs). The tuner times
each candidate with the engine's own CUDA-event kernel timer on the real op
list and keeps the fastest; results are cached per (nstates, ncat, pattern
bucket) for the life of the process. The tile changes speed only: every
candidate computes the same values.
"""
from __future__ import annotations

import math

CANDIDATES = (32, 64, 128)
_cache: dict = {}


def _key(eng):
    return (eng.nstates, eng.ncat, int(math.log2(max(eng.nptn, 1))))


def tune(eng, ops_arr, a, b, length, reps=3):
    """Pick and set the fastest tile for this engine; returns (tile, {tile: ms})."""
    key = _key(eng)
    if key in _cache:
        eng.set_tile(_cache[key][0])
        return _cache[key]
    times = {}
    # tile 1 selects the one-thread-per-pattern kernel of 4-state models
    for tile in ((1,) if eng.nstates == 4 else ()) + CANDIDATES:
        if tile * eng.ncat > 512 and tile > 32:
            continue
        eng.set_tile(tile)
        eng.compute_likelihood(ops_arr, a, b, length)  # warm-up
        eng.set_timing(True)
        for _ in range(reps):
            eng.compute_likelihood(ops_arr, a, b, length)
        ms, n = eng.timing()
        eng.set_timing(False)
        times[tile] = ms / max(n, 1)
    best = min(times, key=times.get)
    eng.set_tile(best)
    _cache[key] = (best, times)
    return best, times
