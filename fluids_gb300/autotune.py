"""Launch-shape autotuner for a context's step.

The threads per block of the step's kernels (sph_set_block_size) are chosen by timing a
few steps of the live context at each candidate and keeping the fastest; for a batched
context the candidates are the shapes of its persistent tile launches -- threads per block
and CTAs per SM (sph_set_tile_shape) of the grid whose warps take the 32-particle scene
tiles.  The choice is
stored in a JSON file keyed by GPU name, method, mode, batched or not, and the particle
count rounded to a power of two, so later contexts of the same kind reuse it without
timing.  The launch shape never changes results (tests/test_autotune.py), only speed.

    from fluids_gb300 import autotune
    choice = autotune.tune(ctx, method=0, mode=1, batched=False)

The file is $SPH_TUNE_CACHE if set, else ~/.cache/fluids_gb300/launch.json.
"""
import json
import math
import os
import time

CANDIDATES = (64, 128, 256)
# CTAs per SM of a batched context's persistent tile launches (0: 2048 / block size)
TILE_CTAS = (0, 2, 4)


def cache_path():
    return os.environ.get("SPH_TUNE_CACHE") or os.path.join(os.path.expanduser("~"), ".cache", "fluids_gb300",
                                                            "launch.json")


def device_name():
    try:
        import torch
        if torch.cuda.is_available():
            return torch.cuda.get_device_name()
    except Exception:
        pass
    return "cuda"


def tune_key(device, method, mode, batched, n):
    bucket = int(math.ceil(math.log2(max(int(n), 1))))
    return "%s|method%d|mode%d|%s|n2^%d" % (device, int(method), int(mode), "batched" if batched else "single",
                                            bucket)


def load_cache(path=None):
    path = path or cache_path()
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def store(key, entry, path=None):
    path = path or cache_path()
    data = load_cache(path)
    data[key] = entry
    os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
    tmp = path + ".tmp%d" % os.getpid()
    with open(tmp, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def measure(ctx, block_size, steps, warmup, clock=time.perf_counter, ctas=None):
    """Seconds per step of ctx at block_size (and, for a batched context, ctas CTAs per SM of
    the tile launches); the state advances by warmup + steps."""
    ctx.set_block_size(block_size)
    if ctas is not None:
        ctx.set_tile_shape(ctas)
    ctx.simulate(warmup)
    ctx.synchronize()
    t0 = clock()
    ctx.simulate(steps)
    ctx.synchronize()
    return (clock() - t0) / max(steps, 1)


# the particle state a step carries to the next one (order, positions, velocities)
STATE_FIELDS = ("POS", "VEL", "VEL_HALF", "ID")


def tune(ctx, method, mode, batched, steps=10, warmup=3, candidates=CANDIDATES, use_cache=True, path=None,
         device=None, clock=time.perf_counter, restore=True):
    """Sets the fastest block size on ctx and returns {block_size, source, seconds_per_step}.
    With restore, the particle state is put back after the timing steps, so a tuned context
    continues from where it was."""
    key = tune_key(device or device_name(), method, mode, batched, ctx.particle_count())
    tiles = batched and hasattr(ctx, "set_tile_shape")
    if use_cache:
        hit = load_cache(path).get(key)
        if hit and hit.get("block_size") in candidates and (not tiles or "ctas_per_sm" in hit):
            ctx.set_block_size(hit["block_size"])
            if tiles:
                ctx.set_tile_shape(hit["ctas_per_sm"])
            return dict(hit, source="cache", key=key)
    saved = {f: ctx.get(f) for f in STATE_FIELDS} if restore and hasattr(ctx, "get") else None
    if tiles:
        shapes = [(int(bs), int(k)) for bs in candidates for k in TILE_CTAS]
        tried = {sh: measure(ctx, sh[0], steps, warmup, clock, ctas=sh[1]) for sh in shapes}
    else:
        tried = {(int(bs), None): measure(ctx, bs, steps, warmup, clock) for bs in candidates}
    if saved is not None:
        for f, a in saved.items():
            ctx.set(f, a)
    best = min(tried, key=lambda sh: (tried[sh], -sh[0], -(sh[1] or 0)))
    ctx.set_block_size(best[0])
    if tiles:
        ctx.set_tile_shape(best[1])
        entry = {"block_size": best[0], "ctas_per_sm": best[1],
                 "seconds_per_step": {"%d/%d" % sh: t for sh, t in sorted(tried.items())}}
    else:
        entry = {"block_size": best[0], "seconds_per_step": {str(sh[0]): t for sh, t in sorted(tried.items())}}
    if use_cache:
        store(key, entry, path)
    return dict(entry, source="timed", key=key)
