"""Autotuner of the device runtime's launch knobs (the reference searched Pluto
tile sizes with a pybench sweep, tests/pluto_tile_test.py:9-54).

Knobs (ofd_set_tuning, ofd_set_persistent, ofd_set_ghost_schedule):
per-sweep kernel (0 TMA-tiled, 1 plain), the x chunking multiplier (CTA
waves), the plain kernel's block shape, persistent stepping (whole steps in
one cooperative launch) and, for the generated space-order-4 ghosts, where
their recompute runs (beside the stress sweep or after it) and its grid.  Each
candidate runs a few profiled steps on a scratch handle of the same shape
(zero fields, constant media: the kernels' cost does not depend on values),
the fastest is kept, and results are cached in a JSON file keyed by grid
dims, space order, storage and media mode.  Results are bit-identical across
knobs, so tuning never changes answers.
"""
import json
import os
import threading

from . import runtime

_lock = threading.Lock()
DEFAULT = {'stress_variant': 0, 'velocity_variant': 0, 'chunk_waves': 1, 'plain_bx': 32, 'plain_by': 8,
           'persistent': 0}
# recompute schedules tried when the configuration has generated ghosts:
# (mode, blocks per SM); the library's default comes first
RC_CANDIDATES = ((1, 4), (1, 2), (0, 8))


def cache_path():
    return os.environ.get('OFD_TUNE_CACHE', os.path.join(os.path.expanduser('~'), '.cache', 'opesci_gb300',
                                                         'autotune.json'))


def _key(cfg, het):
    # size class: dims rounded to multiples of 32 (the knobs vary slowly with size)
    c = [(cfg.dim[i] + 16) // 32 for i in range(3)]
    return 'c%dx%dx%d_so%d_st%d_h%d' % (c[0], c[1], c[2], cfg.space_order, cfg.storage, het)


def _load():
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _save(d):
    p = cache_path()
    os.makedirs(os.path.dirname(p), exist_ok=True)
    tmp = p + '.tmp'
    with open(tmp, 'w') as f:
        json.dump(d, f, indent=1, sort_keys=True)
    os.replace(tmp, p)


def _time(sim, knobs, steps):
    """ms per step of graph (or persistent) stepping, best of two runs."""
    import time
    sim.set_tuning(**knobs)
    sim.step_graph(2)
    sim.sync()
    best = None
    for _ in range(2):
        t0 = time.perf_counter()
        sim.step_graph(steps)
        sim.sync()
        t = (time.perf_counter() - t0) * 1e3 / steps
        best = t if best is None else min(best, t)
    return best


def tune(cfg, ks, kv, het=1, steps=20, use_cache=True):
    """Best knobs for configuration ``cfg`` with literal tables ks/kv."""
    key = _key(cfg, het)
    with _lock:
        cache = _load() if use_cache else {}
        if key in cache:
            return dict(cache[key]['knobs'])
    sim = runtime.Simulation(cfg)
    try:
        sim.set_coefficients(het, ks, kv)
        sim.set_media_const(1e-3, 1.0, 1.0)
        gen = het and sim.set_het_ghost_coefficients()
        results = []
        best = dict(DEFAULT)
        best_t = None
        for sv in (0, 1):
            for vv in (0, 1):
                k = dict(best, stress_variant=sv, velocity_variant=vv)
                t = _time(sim, k, steps)
                results.append((k, t))
                if best_t is None or t < best_t:
                    best, best_t = k, t
        for w in (2, 4):
            k = dict(best, chunk_waves=w)
            t = _time(sim, k, steps)
            results.append((k, t))
            if t < best_t:
                best, best_t = k, t
        if best['stress_variant'] == 1 or best['velocity_variant'] == 1:
            for bx, by in ((64, 4), (32, 4), (128, 2)):
                k = dict(best, plain_bx=bx, plain_by=by)
                t = _time(sim, k, steps)
                results.append((k, t))
                if t < best_t:
                    best, best_t = k, t
        # persistent stepping: all phases of many steps in one launch
        k = dict(best, persistent=1)
        t = _time(sim, k, steps)
        results.append((k, t))
        if t < best_t:
            best, best_t = k, t
        if gen and not best['persistent']:
            for mode, bps in RC_CANDIDATES[1:]:
                k = dict(best, rc_mode=mode, rc_bps=bps)
                t = _time(sim, k, steps)
                results.append((k, t))
                if t < best_t:
                    best, best_t = k, t
    finally:
        sim.close()
    if use_cache:
        with _lock:
            cache = _load()
            cache[key] = {'knobs': best, 'ms_per_step': best_t,
                          'candidates': [[k, t] for k, t in results]}
            _save(cache)
    return best
