"""Autotuner for the launch parameters of the CUDA path.

Tunes, by timing real steps on the current GPU:

* batched Cahn-Hilliard (``BatchTuning``): stencil tile shape, x planes per
  work item, persistent blocks per SM, cuFFT batch grouping, steps per
  captured CUDA graph;
* forward-Euler finite differences: steps fused per HBM pass (1, 2, 4);
* single-grid Cahn-Hilliard: stencil tile shape.

Search is coordinate descent from the defaults (one knob at a time, keep the
fastest value).  Results are cached in a JSON file keyed by GPU name and a
signature of the workload (``EVX_AUTOTUNE_CACHE`` overrides the path; the
default is ``~/.cache/evoxels_gb300/autotune.json``).  Every tuned choice gives
the same results up to the FFT grouping's float32 rounding.
"""

from __future__ import annotations

import dataclasses
import hashlib
import json
import os
import threading

import numpy as np
import torch

from . import _lib

_lock = threading.Lock()


def cache_path():
    return os.environ.get("EVX_AUTOTUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "evoxels_gb300", "autotune.json"))


def _load():
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(key, value):
    with _lock:
        d = _load()
        d[key] = value
        p = cache_path()
        os.makedirs(os.path.dirname(p), exist_ok=True)
        tmp = p + ".tmp"
        with open(tmp, "w") as f:
            json.dump(d, f, indent=1, sort_keys=True)
        os.replace(tmp, p)


def _key(kind, sig):
    gpu = torch.cuda.get_device_name(torch.cuda.current_device())
    h = hashlib.sha1(json.dumps(sig, sort_keys=True).encode()).hexdigest()[:16]
    return f"{kind}|{gpu}|{h}"


def time_cuda(fn, reps=3, warmup=1):
    """Median milliseconds of ``fn()`` with CUDA events on the current stream."""
    for _ in range(warmup):
        fn()
    st = torch.cuda.current_stream()
    times = []
    for _ in range(reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(st)
        fn()
        b.record(st)
        b.synchronize()
        times.append(a.elapsed_time(b))
    return float(np.median(times))


def _descend(start: dict, space: dict, measure):
    """Coordinate descent: for each knob try its values, keep the fastest."""
    best = dict(start)
    best_t = measure(best)
    log = [(dict(best), best_t)]
    for knob, values in space.items():
        for v in values:
            if v == best[knob]:
                continue
            cand = dict(best, **{knob: v})
            t = measure(cand)
            log.append((dict(cand), t))
            if t < best_t:
                best, best_t = cand, t
    return best, best_t, log


BATCH_SPACE = {
    "tile_variant": [-1, 0, 1],
    "x_chunk": [0, 8, 32, 64],
    "graph_steps": [20, 0, 50],
    "fft_group_max": [0, 4, 1],
    "blocks_per_sm": [0, 2],
}


def tune_batched(shapes, D=1.0, eps=3.0, dt=0.1, mu_hom=None, steps=10, use_cache=True, space=None):
    """Best ``BatchTuning`` for these instances (timed forward steps)."""
    from .batched import BatchedCahnHilliard, BatchTuning
    sig = {"shapes": sorted([list(s) for s in shapes]), "steps": steps}
    key = _key("batched", sig)
    if use_cache:
        hit = _load().get(key)
        if hit:
            return BatchTuning(**hit["tuning"])
    rng = np.random.default_rng(0)
    fields = [0.5 + 0.1 * rng.random(s) for s in shapes]
    space = space or BATCH_SPACE

    def measure(cfg):
        b = BatchedCahnHilliard(shapes, D, eps, dt, mu_hom=mu_hom, tuning=BatchTuning(**cfg))
        u = b.pack(fields)
        return time_cuda(lambda: b.forward(u, steps))

    best, best_t, log = _descend(dataclasses.asdict(BatchTuning()), space, measure)
    _store(key, {"tuning": best, "ms": best_t, "tried": [[c, t] for c, t in log]})
    return BatchTuning(**best)


def tune_fd_steps_per_pass(problem, dt, u, steps=8, use_cache=True):
    """Fastest steps-per-pass (1, 2, 4) of forward Euler for this grid and BCs."""
    from .timesteppers import ForwardEuler
    sig = {"shape": list(problem.vg.shape), "bc": repr(problem.bc), "steps": steps}
    key = _key("fd_spp", sig)
    if use_cache:
        hit = _load().get(key)
        if hit:
            return int(hit["steps_per_pass"])
    times = {}
    for spp in (1, 2, 4):
        st = ForwardEuler(problem, dt, steps_per_pass=spp)
        times[spp] = time_cuda(lambda: st.advance(u, steps))
    best = min(times, key=times.get)
    _store(key, {"steps_per_pass": best, "ms": times})
    return best


def tune_tile_variant(stepper, u, steps=4, use_cache=True):
    """Fastest stencil tile shape for a single-grid IMEX stepper; sets it and returns it."""
    L = _lib.lib()
    sig = {"shape": list(stepper.problem.vg.shape), "steps": steps}
    key = _key("tile", sig)
    if use_cache:
        hit = _load().get(key)
        if hit:
            L.evx_set_tile_variant(int(hit["variant"]))
            return int(hit["variant"])
    times = {}
    for v in (0, 1):
        L.evx_set_tile_variant(v)
        times[v] = time_cuda(lambda: stepper.advance(u, steps))
    best = min(times, key=times.get)
    L.evx_set_tile_variant(best)
    _store(key, {"variant": best, "ms": times})
    return best
