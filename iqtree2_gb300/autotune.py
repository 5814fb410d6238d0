"""Schedule and pattern-tile autotuner for the mixed-precision traversal.

Candidates: the fused schedule (one launch walks the op list per pattern
tile) and the level-synchronous schedule (one launch per tree level), each
with 32/64/128 patterns per CTA, plus the one-thread-per-pattern kernel for
4-state models. The best choice depends on the state count (registers per
thread), the category count, the number of patterns (how many CTAs fill the
152 SMs) and the tree's depth. The tuner times each candidate with the
engine's CUDA-event kernel timer on the real op list and keeps the fastest;
results are cached per (nstates, ncat, pattern bucket, op count) for the life
of the process. Every candidate computes the same values.
"""
from __future__ import annotations

import math

TILES = (32, 64, 128)
_cache: dict = {}


def candidates(eng):
    out = [(1, 0)] if eng.nstates == 4 and eng.ncat <= 4 else []
    for sched in (0, 1):
        for tile in TILES:
            if tile > 32 and tile * eng.ncat > 512:
                continue
            out.append((tile, sched))
    return out


def tune(eng, ops_arr, a, b, length, reps=3):
    """Pick and set the fastest (tile, schedule); returns (label, {label: ms})."""
    key = (eng.nstates, eng.ncat, int(math.log2(max(eng.nptn, 1))), len(ops_arr))
    if key in _cache:
        (tile, sched), times = _cache[key]
        eng.set_tile(tile)
        eng.set_schedule(sched)
        return f"{tile}/{'level' if sched else 'fused'}", times
    times, best, best_ms = {}, None, float("inf")
    for tile, sched in candidates(eng):
        eng.set_tile(tile)
        eng.set_schedule(sched)
        eng.compute_likelihood(ops_arr, a, b, length)  # warm-up
        eng.set_timing(True)
        for _ in range(reps):
            eng.compute_likelihood(ops_arr, a, b, length)
        ms, n = eng.timing()
        eng.set_timing(False)
        ms /= max(n, 1)
        times[f"{tile}/{'level' if sched else 'fused'}"] = ms
        if ms < best_ms:
            best, best_ms = (tile, sched), ms
    eng.set_tile(best[0])
    eng.set_schedule(best[1])
    _cache[key] = (best, times)
    return f"{best[0]}/{'level' if best[1] else 'fused'}", times
