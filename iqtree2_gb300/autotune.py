"""Schedule and pattern-tile autotuner for the mixed-precision traversal.

Candidates: the fused schedule (one launch walks the op list per pattern
tile) and the level-synchronous schedule (one launch per tree level), each
with 32/64/128 patterns per CTA, plus the one-thread-per-pattern kernel for
4-state models; on the tensor-core path (split TF32) the tile is the MMA's
128 rows and only the schedule is tuned. The best choice depends on the state count (registers per
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
    """(tile, schedule, stages, kpieces) tuples; stages and kpieces only matter
    on the tensor-core path; schedule 0 = fused, 1 = level-synchronous,
    2 = dataflow (4-state one-thread-per-pattern kernel), 3 = level-synchronous
    with the warp-specialised tensor-core kernel, 4 = level-synchronous with
    operand A in tensor memory (20 states, split TF32), 5 = as 3 with
    category-split items on the narrow levels (up to 32 padded states),
    6 = dataflow on the tensor cores (one launch of category-split items,
    each waiting for the items writing its children), 7 = as 6 with whole
    (op, tile) items, 8 = level-synchronous on the deep-ring kernel (20 states,
    split TF32: one CTA per SM, six categories in flight, operand A in tensor
    memory; one-op levels on the CUDA-core tail), 9 = as 8 with the one-op
    levels in one launch of the same kernel, each CTA taking its tiles through
    all of them."""
    if getattr(eng, "tensor_cores", False):  # one CTA = 128 patterns (the MMA's M)
        npad = (eng.nstates + 3) // 4 * 4
        pieces = (1, 2) if (npad > 32 and npad % 16 == 0) else (1,)
        out = [(0, sched, st, kp) for sched in (0, 1, 3) for st in (2, 3, 4) for kp in pieces]
        if npad <= 32:  # category-split narrow levels on the tensor cores
            out += [(0, 5, st, 1) for st in (2, 3)]
        out += [(0, 6, st, kp) for st in (2, 3) for kp in pieces]  # dataflow, category-split items
        if npad > 32 and npad % 16 == 0:  # ... with K in quarters and one accumulator buffer
            out += [(0, 6, st, 4) for st in (2, 3)]
        out += [(0, 7, 2, kp) for kp in pieces]  # dataflow, whole (op, tile) items
        if npad == 20 and getattr(eng, "precision", 0) == 2:  # split TF32
            out.append((0, 4, 0, 0))
            out += [(0, 8, 0, 0), (0, 9, 0, 0)]  # deep ring, one CTA per SM
        return out
    out = ([(1, 0, 0, 0), (1, 1, 0, 0), (1, 2, 0, 0), (2, 1, 0, 0)]
           if eng.nstates == 4 and eng.ncat <= 4 else [])
    for sched in (0, 1):
        for tile in TILES:
            if tile > 32 and tile * eng.ncat > 512:
                continue
            out.append((tile, sched, 0, 0))
    return out


def label(cand):
    tile, sched, stages, kp = cand
    names = ('fused', 'level', 'flow', 'level-ws', 'level-tm', 'level-wsc', 'flow-tc', 'flow-tcw', 'level-ring',
             'level-ring-all')
    return (f"{tile}/{names[sched]}" +
            (f"/s{stages}" if stages else "") +
            (f"/k{kp}" if kp else ""))


def apply(eng, cand):
    tile, sched, stages, kp = cand
    eng.set_tile(tile)
    eng.set_schedule(sched)
    eng.set_stages(stages)
    eng.set_kpieces(kp)


def tune(eng, ops_arr, a, b, length, reps=3):
    """Pick and set the fastest candidate; returns (label, {label: ms})."""
    key = (eng.nstates, eng.ncat, int(math.log2(max(eng.nptn, 1))), len(ops_arr), getattr(eng, "precision", 1))
    if key in _cache:
        best, times = _cache[key]
        apply(eng, best)
        return label(best), times
    times, best, best_ms = {}, None, float("inf")
    for cand in candidates(eng):
        apply(eng, cand)
        eng.compute_likelihood(ops_arr, a, b, length)  # warm-up
        eng.set_timing(True)
        for _ in range(reps):
            eng.compute_likelihood(ops_arr, a, b, length)
        ms, n = eng.timing()
        eng.set_timing(False)
        ms /= max(n, 1)
        times[label(cand)] = ms
        if ms < best_ms:
            best, best_ms = cand, ms
    apply(eng, best)
    _cache[key] = (best, times)
    return label(best), times
