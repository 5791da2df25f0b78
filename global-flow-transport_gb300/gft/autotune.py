"""Autotuner of the library's launch-configuration knobs (gft_set_knob).

The knobs change only how kernels are launched -- the raymarch kernels' grid
(one block per pixel tile, or a persistent grid of a few blocks per SM, which
bounds how many tiles are in flight and so the set of gradient lines the
adjoint's reductions keep in L2), the grid of the gradient's weight pass
alone (which runs ahead on a side stream beside the forward kernels; a small
persistent grid leaves them room), whether the weight pass instead runs
camera by camera beside the adjoint's scatter (the library's side stream),
the block size of the advection and
SampleGridTransform kernels, and the segment count of the transmittance scans
-- never what they compute.  ``tune`` times a step for every candidate of
every knob with CUDA events on the current stream (a coordinate search: each
knob in turn, the others at their best so far) and keeps the fastest; results
are cached per workload key (shapes, views, storage type, gradient mode and
device) in memory and, when the environment variable GFT_TUNE_CACHE names a
file, in that JSON file.

Knob values are process-wide and read when a launch is issued, so a step
captured into a CUDA graph keeps the values set at its capture.
"""
import json
import os
import time

import numpy as np
import torch

from . import _lib

# name -> (knob id of gft.h, candidates, default)
KNOBS = {
    'weights_pipeline': (5, (0, 1), 0),
    'raymarch_blocks_per_sm': (0, (0, 2, 3, 4, 6), 0),
    'advect_threads': (1, (256, 128, 64), 256),
    'resample_threads': (2, (256, 128, 64), 256),
    'scan_segments': (3, (8, 4, 16), 8),
    'weights_blocks_per_sm': (4, (0, 2, 4, 6, 8), 0),
}

_cache = {}


def set_knob(name, value):
    knob = KNOBS[name][0]
    _lib.check(_lib.load().gft_set_knob(knob, int(value)), 'gft_set_knob(%s, %s)' % (name, value))


def get_knob(name):
    return int(_lib.load().gft_get_knob(KNOBS[name][0]))


def knobs():
    """The current value of every knob."""
    return {name: get_knob(name) for name in KNOBS}


def apply(values):
    for name, v in values.items():
        set_knob(name, v)


def defaults():
    return {name: d for name, (_, _, d) in KNOBS.items()}


class knob_settings:
    """Context manager: the given knob values inside, the previous ones after."""

    def __init__(self, values):
        self.values = dict(values)

    def __enter__(self):
        self.prev = knobs()
        apply(self.values)
        return self

    def __exit__(self, *a):
        apply(self.prev)


def _load_file():
    path = os.environ.get('GFT_TUNE_CACHE')
    if path and os.path.exists(path):
        try:
            with open(path) as f:
                return json.load(f)
        except (OSError, ValueError):
            return {}
    return {}


def _store_file(key, values):
    path = os.environ.get('GFT_TUNE_CACHE')
    if not path:
        return
    data = _load_file()
    data[key] = values
    tmp = path + '.tmp'
    with open(tmp, 'w') as f:
        json.dump(data, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def time_ms(fn, reps=5, warmup=2):
    """Median milliseconds of fn() with CUDA events on the current stream."""
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
    for a, b in evs:
        a.record()
        fn()
        b.record()
    torch.cuda.synchronize()
    return float(np.median([a.elapsed_time(b) for a, b in evs]))


def tune(fn, key=None, names=None, reps=5, warmup=2, log=None):
    """Coordinate search over the knobs ``names`` (all by default) for the
    fastest fn(); applies and returns the chosen values (and caches them under
    ``key``).  ``log`` (a dict) receives the timings of every candidate."""
    if key is not None:
        if key in _cache:
            apply(_cache[key])
            return dict(_cache[key])
        stored = _load_file().get(key)
        if stored:
            _cache[key] = stored
            apply(stored)
            return dict(stored)
    t0 = time.perf_counter()
    best = knobs()
    for name in (names or list(KNOBS)):
        times = {}
        for v in KNOBS[name][1]:
            set_knob(name, v)
            times[v] = time_ms(fn, reps, warmup)
        best[name] = min(times, key=times.get)
        set_knob(name, best[name])
        if log is not None:
            log[name] = {str(k): round(t, 4) for k, t in times.items()}
    if log is not None:
        log['seconds'] = time.perf_counter() - t0
    if key is not None:
        _cache[key] = dict(best)
        _store_file(key, best)
    return best


def step_key(step):
    """Workload key of a gft.pipeline step: grid, views, images, samples,
    shadow frustum, storage type, gradient mode, device name."""
    from . import ops
    dev = torch.cuda.get_device_name(step.dev)
    res = getattr(step, 'res', None)
    shapes = getattr(step, 'shapes', None)
    views = ('x'.join(map(str, res)) + '*%d' % len(step.cams)) if res is not None else 'views%d' % len(shapes)
    return '|'.join([type(step).__name__, 'x'.join(map(str, step.shape)), views,
                     'x'.join(map(str, step.shadow_res)), str(step.storage_dtype), ops.get_grad_mode(), dev])
