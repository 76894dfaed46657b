"""Launch-parameter autotuner with a JSON cache.

Knobs (yv_launch_config): threads per block, the register budget of the
persistent kernel (resident blocks per SM: more blocks = fewer registers and
a shallower register-resident state), top-of-tree nodes staged in shared
memory (0 / 73 / 585 = 0 / 3 / 4 full levels) and rays a warp takes per
refill (the per-lane work granularity).  Each candidate is timed with CUDA
events (median of `reps` after one warm-up); the winner is cached per device
and workload signature in $YOXEL_AUTOTUNE_CACHE (default
~/.cache/yoxel/autotune.json).
"""
import itertools
import json
import os

DEFAULT_CACHE = os.path.join(os.path.expanduser("~"), ".cache", "yoxel", "autotune.json")

SVO_SPACE = dict(block_threads=[128, 256], blocks_per_sm=[3, 4, 5], smem_nodes=[0, 73, 585],
                 tile_rays=[24, 32])
BATCH_SPACE = dict(block_threads=[128, 256], blocks_per_sm=[2, 3, 4])


def _cache_path():
    return os.environ.get("YOXEL_AUTOTUNE_CACHE", DEFAULT_CACHE)


def _load():
    try:
        with open(_cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(cache):
    p = _cache_path()
    try:
        os.makedirs(os.path.dirname(p), exist_ok=True)
        tmp = p + ".tmp"
        with open(tmp, "w") as f:
            json.dump(cache, f, indent=1, sort_keys=True)
        os.replace(tmp, p)
    except OSError:
        pass  # a read-only home only disables caching


def device_key():
    import torch
    p = torch.cuda.get_device_properties(torch.cuda.current_device())
    return f"{p.name}|sm{p.major}{p.minor}|{p.multi_processor_count}"


def tune(key, space, apply, run, reps=3, use_cache=True, flush=None):
    """Times every configuration of `space` (dict of lists): apply(cfg) then
    run() per trial.  Returns (best cfg, {cfg-json: ms}).  `flush` (optional)
    runs before each timed trial, outside the events."""
    import torch
    full_key = device_key() + "|" + key
    cache = _load() if use_cache else {}
    if use_cache and full_key in cache:
        best = cache[full_key]["best"]
        apply(best)
        return best, cache[full_key].get("times", {})
    names = list(space)
    times = {}
    best, best_ms = None, float("inf")
    for values in itertools.product(*[space[n] for n in names]):
        cfg = dict(zip(names, values))
        apply(cfg)
        run()
        torch.cuda.synchronize()
        ts = []
        for _ in range(reps):
            if flush is not None:
                flush()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record()
            run()
            b.record()
            torch.cuda.synchronize()
            ts.append(a.elapsed_time(b))
        ts.sort()
        ms = ts[len(ts) // 2]
        times[json.dumps(cfg, sort_keys=True)] = ms
        if ms < best_ms:
            best, best_ms = cfg, ms
    apply(best)
    if use_cache:
        cache[full_key] = {"best": best, "ms": best_ms, "times": times}
        _store(cache)
    return best, times


def tune_renderer(renderer, key, out=None, reps=3, use_cache=True, flush=None, space=None):
    """Autotunes an SVO Renderer's launch configuration for its current scene."""
    import torch
    w, h = renderer.GetResolution()
    if out is None:
        out = torch.empty((h, w), dtype=torch.int32, device="cuda")
    return tune("svo|" + key, space or SVO_SPACE, lambda c: renderer.SetLaunchConfig(**c),
                lambda: renderer.render_async(rgba=out), reps, use_cache, flush)


def tune_batch(batch, key, reps=3, use_cache=True, flush=None, space=None, graph=True):
    return tune("batch|" + key, space or BATCH_SPACE, lambda c: batch.set_launch_config(**c),
                lambda: batch.render(graph=graph), reps, use_cache, flush)
