"""Autotuner for plan launch parameters.

The reference fixes its launch configuration in jinja2 templates
(neato.py:160-163: one thread per even row, one block per system).  Here the
launch parameters of a plan are searched by timing on the current GPU and
cached per (device, kernel family, n, precision, layout):

  f64_x_variant  contiguous FP64 sweeps: transposing tile ring / whole-system
                 shared tile (threads per system = 1 in both)
  f64_threads    threads per block of the one-thread-per-system FP64 kernel
                 (systems per block for the strided sweeps)
  refine_w       warps per CTA of the FP32 + refinement kernel (4, 8, 16;
                 threads per system = 32, rows per lane = n / 32 in registers)
  refine_spw     systems per warp (2 stages twice as many adjacent systems
                 per CTA: wider row segments for strided y/z sweeps)
  refine_kernel  n = 512: the paired-chunk TMA kernels (16 rows per
                 thread, two 8-row halves per packed FP32x2 instruction;
                 refine_w = systems per CTA of contiguous layouts) with one
                 strided group per CTA (2) or persistent strided CTAs (3);
                 1 the chunked kernel (refine_w, refine_spw as above)
  refine_prefetch  one-group strided CTAs: L2 prefetch of the tile needed
                 p / 2 waves later (p = 1, 2, 3 searched; 0 and 4, no
                 prefetch and two waves, measured slower on every axis)
  refine_tps     threads per system: 32 everywhere (paired-chunk kernels:
                 16 rows per thread; chunked kernel: one warp per system);
                 for 512 < n <= 1024 also 64 (two overlapping 512-row
                 windows, 16 rows per lane, instead of one warp with 32)

Usage:
    best = autotune.tune(plan, run, key)   # run() launches the workload once
    autotune.apply_cached(plan, key)       # reuse a previous result
The cache is a JSON file at $NTK_AUTOTUNE_CACHE, default
~/.cache/ntk/autotune.json.
"""
import json
import os
import threading

_lock = threading.Lock()

SPACE = {
    "fp64": [{"f64_x_variant": [0, 1], "f64_threads": [64, 128]}],
    "fp32": [{"refine_kernel": [2], "refine_w": [4, 8, 16], "refine_prefetch": [1, 2, 3]},
             {"refine_kernel": [3], "refine_w": [4, 8, 16]},
             {"refine_kernel": [1], "refine_w": [4, 8, 16], "refine_spw": [1, 2]}],
    "fp32_refine": [{"refine_kernel": [2], "refine_w": [4, 8, 16], "refine_prefetch": [1, 2, 3]},
                    {"refine_kernel": [3], "refine_w": [4, 8, 16]},
                    {"refine_kernel": [1], "refine_w": [4, 8, 16], "refine_spw": [1, 2]}],
}
# a refinement CTA stages at most 16 systems (refine_w * refine_spw)
MAX_GROUP = 16


def cache_path():
    return os.environ.get("NTK_AUTOTUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "ntk", "autotune.json"))


def _load():
    try:
        with open(cache_path()) as fh:
            return json.load(fh)
    except (OSError, ValueError):
        return {}


def _store(data):
    path = cache_path()
    os.makedirs(os.path.dirname(path), exist_ok=True)
    tmp = path + ".tmp%d" % os.getpid()
    with open(tmp, "w") as fh:
        json.dump(data, fh, indent=1, sort_keys=True)
    os.replace(tmp, path)


def device_name():
    import torch

    return torch.cuda.get_device_name(torch.cuda.current_device())


def cache_key(plan, key):
    return "|".join([device_name(), str(plan.n), str(plan.precision), str(key)])


def candidates(precision, n=None):
    """The configurations searched for a plan of this precision and system
    length n (threads per system: 64 only offered for 512 < n <= 1024)."""
    out = []
    for space in SPACE.get(precision, [{}]):
        if "refine_kernel" in space:
            tps = [32, 64] if (n is not None and 512 < n <= 1024 and space["refine_kernel"] == [1]) else [32]
            space = dict(space, refine_tps=tps)
        configs = [{}]
        for name, values in space.items():
            configs = [dict(c, **{name: v}) for c in configs for v in values]
        out += [c for c in configs if c.get("refine_w", 1) * c.get("refine_spw", 1) <= MAX_GROUP]
    return out


def _time(run, repeats, timer):
    if timer is not None:
        return timer(run, repeats)
    import torch

    run()  # warm-up (and plan tables)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(repeats):
        run()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / repeats


def tune(plan, run, key, repeats=5, timer=None, use_cache=True):
    """Time every candidate configuration of plan's precision with run(),
    apply the fastest, cache and return {"config": ..., "ms": ..., "all": ...}."""
    ck = cache_key(plan, key)
    if use_cache:
        with _lock:
            hit = _load().get(ck)
        if hit:
            plan.set_tuning(**hit["config"])
            return hit
    results = []
    for cfg in candidates(plan.precision, getattr(plan, "n", None)):
        plan.set_tuning(**cfg)
        results.append((_time(run, repeats, timer), cfg))
    results.sort(key=lambda r: r[0])
    best_ms, best = results[0]
    plan.set_tuning(**best)
    entry = {"config": best, "ms": best_ms, "all": [{"config": c, "ms": m} for m, c in results]}
    with _lock:
        data = _load()
        data[ck] = entry
        _store(data)
    return entry


def apply_cached(plan, key):
    """Apply a cached configuration for (plan, key); returns it or None."""
    with _lock:
        hit = _load().get(cache_key(plan, key))
    if hit:
        plan.set_tuning(**hit["config"])
        return hit["config"]
    return None
