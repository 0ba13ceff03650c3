"""Launch-shape tuner of the sweep kernel.

The sweep can run with different block sizes (threads per block = how many
cell-aligned 32-particle chunks a block holds), queue depths (neighbours each
thread stages before the pair arithmetic) and persistent-grid sizes (blocks
per SM).  Every choice gives the same results; the fastest depends on the
GPU and on the case (particles per cell, wall fraction, batch size).
:func:`autotune` times each candidate on the live case with a few steps and
keeps the fastest; the choice is cached per (GPU, case signature) in a JSON
file so later runs of the same configuration skip the search.
"""
from __future__ import annotations

import json
import os
import time

from . import _lib

# (variant, threads per block, queued neighbours per thread, the most
# resident warps per SM its register budget allows); the variant numbers are
# those of aqua_set_tuning (3 and 4 stage the candidates with bulk copies,
# 5 and 6 sum each candidate group directly, without a queue, 7 and 8 too,
# with the next group prefetched by asynchronous copies, 9-14 those
# compiled for 28, 32 or 36 resident warps per SM)
VARIANTS = ((0, 128, 128, 24), (1, 64, 128, 24), (2, 64, 64, 24),
            (3, 64, 128, 24), (4, 64, 64, 24), (5, 64, 0, 24), (6, 128, 0, 24),
            (7, 64, 0, 24), (8, 128, 0, 24), (9, 64, 0, 28), (10, 128, 0, 28),
            (11, 64, 0, 32), (12, 128, 0, 32), (13, 64, 0, 36),
            (14, 128, 0, 36))
# resident warps per SM tried for each variant (blocks = warps * 32 / threads)
WARPS_PER_SM = (8, 12, 16, 20, 24, 28, 32, 36)
MAX_BLOCKS_PER_SM = 32
# the clustered sweep of the fast 3-D build (BIe walls, midpoint scheme):
# (variant, threads per block, blocks per SM tried); 15 and 17 hold at most
# 2 blocks per SM, 16 at most 3 (shared memory, registers)
CLUSTERED = ((15, 256, (1, 2)), (16, 256, (1, 2, 3)), (17, 384, (1, 2)))


def cache_path() -> str:
    return os.environ.get(
        "AQUA_TUNE_CACHE",
        os.path.join(os.path.expanduser("~"), ".cache", "aquagpusph_gb300",
                     "tuning.json"))


def gpu_name() -> str:
    try:
        import torch
        if torch.cuda.is_available():
            return torch.cuda.get_device_name(torch.cuda.current_device())
    except Exception:
        pass
    return "cuda"


def signature(solver, fast: bool) -> str:
    p = solver.params
    n_cases = getattr(solver, "n_cases", 1)
    # particle counts bucketed to 1/16 of a power of two
    n = max(solver.N, 1)
    bucket = 1 << (n.bit_length() - 1)
    bucket = bucket + ((n - bucket) // (bucket // 16 or 1)) * (bucket // 16 or 1)
    return (f"{gpu_name()}|dims={p.dims}|N~{bucket}|cases={n_cases}|"
            f"h={p.h:.6g}|{'fast' if fast else 'exact'}")


def _load():
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _save(d):
    path = cache_path()
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        tmp = path + ".tmp"
        with open(tmp, "w") as f:
            json.dump(d, f, indent=1, sort_keys=True)
        os.replace(tmp, path)
    except OSError:
        pass


def clustered_applies(solver, fast: bool) -> bool:
    """The clustered sweep runs for the fast build in 3-D with BIe walls and
    the midpoint scheme."""
    p = solver.params
    return bool(fast and p.dims == 3 and getattr(p, "boundary", 0) == 0 and
                getattr(p, "scheme", 0) == 0)


def candidates(clustered: bool = False):
    for v, threads, queue, most in VARIANTS:
        for w in WARPS_PER_SM:
            if w > most:
                continue
            b = w * 32 // threads
            if b * threads == w * 32 and 1 <= b <= MAX_BLOCKS_PER_SM:
                yield v, b
    if clustered:
        for v, threads, blocks in CLUSTERED:
            for b in blocks:
                yield v, b


def autotune(solver, fast: bool, steps: int = 3, use_cache: bool = True,
             stream=None) -> dict:
    """Picks the fastest sweep launch shape for the solver's resident case
    and applies it.  Advances the resident state by the timed steps (call it
    during warm-up, or restore the state afterwards)."""
    key = signature(solver, fast)
    cache = _load() if use_cache else {}
    if key in cache:
        v, b = cache[key]["variant"], cache[key]["blocks_per_sm"]
        solver.set_tuning(v, b)
        return dict(cache[key], cached=True)
    results = []
    for v, b in candidates(clustered_applies(solver, fast)):
        try:
            solver.set_tuning(v, b)
        except _lib.AquaError:
            continue
        solver.step(1, graph=True, stream=stream)      # capture + warm
        solver.scalars(stream)
        t0 = time.perf_counter()
        solver.step(steps, graph=True, stream=stream)
        solver.scalars(stream)                         # synchronises
        dt = (time.perf_counter() - t0) / steps
        results.append((dt, v, b))
    solver.check(stream)
    results.sort()
    best_dt, v, b = results[0]
    solver.set_tuning(v, b)
    threads = dict((x[0], x[1]) for x in VARIANTS + CLUSTERED)
    entry = {"variant": v, "blocks_per_sm": b,
             "threads": threads[v],
             "queue": dict((x[0], x[2]) for x in VARIANTS).get(v, 0),
             "ms_per_step": 1e3 * best_dt,
             "candidates": [[round(1e3 * d, 4), vv, bb] for d, vv, bb in results]}
    if use_cache:
        cache[key] = entry
        _save(cache)
    return dict(entry, cached=False)
