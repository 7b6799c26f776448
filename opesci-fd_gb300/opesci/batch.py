"""Batched forward modelling of many independent shots on one GPU.

A shot is an elastic forward model of the layered kind (``layered_problem``):
its own cubic grid, space order, seeded medium, Ricker source and step
count.  Shots are built without the symbolic frontend: heterogeneous update
expressions have literals r_i dt/h, so their tables come from the stored unit
tables (cuda_gen.het_tables) and equal what the frontend would print.

Two batched executions keep every admitted shot resident in HBM:

* grouped (run_grouped): the shots of one space order form a group
  (ofd_group); each phase of a time step is ONE launch over every shot of
  the group, the time loop a replayed two-step CUDA graph, so the GPU is
  filled with CTAs of all shots at once and small shots cost no launches of
  their own;
* streams (run_batched): each shot on its own stream with its own captured
  graph and autotuned launch knobs, slices enqueued round-robin.

The baseline runs the same shots one after another with plain per-kernel
launches.

    python -m opesci.batch --shots 256 [--seed 0]

prints a JSON object with the three aggregate GLUP/s figures.
"""
import argparse
import json
import math
import os
import time

import numpy as np

from . import runtime, autotune
from .models import layered_media, cfl_dt, ricker
from .templates import cuda_gen
from .util import staggered_weights

_WEIGHTS = {}


def _weights(so):
    if so not in _WEIGHTS:
        _WEIGHTS[so] = [float(w) for w in staggered_weights(so)]
    return _WEIGHTS[so]


class Shot(object):
    """One shot: interior edge n, space order, steps, media seed, Ricker peak
    frequency, spacing h (metres)."""

    def __init__(self, n, space_order, steps, seed, f0, h=10.0):
        self.n, self.so, self.steps, self.seed, self.f0, self.h = n, space_order, steps, seed, f0, h

    @property
    def lups(self):
        return float(self.n) ** 3 * self.steps

    def build(self):
        """(ofd_config, media, source index, wavelet, ks, kv) — the same
        problem layered_problem(n, so, steps, seed, f0) builds symbolically."""
        m = self.so // 2
        dims = (self.n + 2 * m,) * 3
        rho, vp, vs = layered_media(dims, seed=self.seed)
        dt = cfl_dt(self.h, float(vp.max()), self.so)
        rng = np.random.default_rng(self.seed + 7919)
        src = tuple(int(v) for v in rng.integers(m + self.n // 4, m + 3 * self.n // 4, size=3))
        wav = ricker(self.steps, dt, self.f0)
        algo = 'levander' if self.so == 4 else 'robertsson'
        cfg = runtime.make_config(dims, self.so, [self.h] * 3, dt, _weights(self.so), storage='f32',
                                  free_surface=[algo] * 6)
        ks, kv = cuda_gen.het_tables(self.so, dt, self.h)
        return cfg, (rho, vp, vs), src, wav, ks, kv

    def to_dict(self):
        return {'n': self.n, 'space_order': self.so, 'steps': self.steps, 'seed': self.seed, 'f0': self.f0}


def make_shots(count=256, seed=0, edge_range=(32, 192), so_choices=(4, 8), f_range=(8.0, 25.0),
               steps_range=(300, 1500)):
    """Seeded shot list: edge log-uniform in edge_range, space order drawn from
    so_choices, Ricker 8-25 Hz, 300-1500 steps, a media seed per shot."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        n = int(round(math.exp(rng.uniform(math.log(edge_range[0]), math.log(edge_range[1])))))
        so = int(rng.choice(so_choices))
        steps = int(rng.integers(steps_range[0], steps_range[1] + 1))
        f0 = float(rng.uniform(*f_range))
        out.append(Shot(n, so, steps, seed * 100003 + i, f0))
    return out


def prepare(shot, tuned=True, built=None):
    cfg, media, src, wav, ks, kv = built if built is not None else shot.build()
    sim = runtime.Simulation(cfg)
    sim.set_coefficients(1, ks, kv)
    sim.set_het_ghost_coefficients()
    sim.set_media(*media)
    sim.set_source(src, wav)
    if tuned:
        sim.set_tuning(**autotune.tune(cfg, ks, kv, het=1))
    return sim


def run_one_by_one(shots, keep=None, built=None):
    """Each shot alone: set up, run with per-kernel launches, wait, free.
    ``built`` holds the shots' prebuilt inputs (Shot.build())."""
    built = built if built is not None else [s.build() for s in shots]
    t0 = time.perf_counter()
    outs = {}
    for i, s in enumerate(shots):
        sim = prepare(s, tuned=False, built=built[i])
        sim.step(s.steps)
        sim.sync()
        if keep is not None and i in keep:
            outs[i] = {f: sim.download(f) for f in runtime.FIELDS}
        sim.close()
    return time.perf_counter() - t0, outs


def run_batched(shots, budget_bytes=150e9, keep=None, built=None, slice_steps=64):
    """All shots resident (admitted in order while their footprint fits the
    budget).  Graph replays are enqueued in slices of ``slice_steps`` steps,
    round-robin over the shots, largest remaining work first, so every
    hardware queue interleaves many shots instead of running them back to
    back; then one wait."""
    built = built if built is not None else [s.build() for s in shots]
    t0 = time.perf_counter()
    pending = list(enumerate(shots))
    outs = {}
    while pending:
        group, used = [], 0
        while pending:
            i, s = pending[0]
            fp = _footprint(s)
            if group and used + fp > budget_bytes:
                break
            pending.pop(0)
            group.append((i, s))
            used += fp
        # set up shots one by one and give each its first slice at once, so
        # the GPU works on earlier shots while later ones are being set up
        sims, rem = [], {}
        for i, s in sorted(group, key=lambda t: -t[1].lups):
            sim = prepare(s, built=built[i])
            k = min(slice_steps, s.steps)
            sim.step_graph(k)
            rem[i] = s.steps - k
            sims.append((i, s, sim))
        while any(rem.values()):
            for i, s, sim in sims:
                k = min(slice_steps, rem[i])
                if k:
                    sim.step_graph(k)
                    rem[i] -= k
        for i, s, sim in sims:
            sim.sync()
            if keep is not None and i in keep:
                outs[i] = {f: sim.download(f) for f in runtime.FIELDS}
            sim.close()
    return time.perf_counter() - t0, outs


_last_prepare_s = [0.0]   # host setup time of the last run_grouped call (handles, media, sources)


def run_grouped(shots, budget_bytes=150e9, keep=None, built=None, chunk_planes=0):
    """All shots resident (admitted in order while their footprint fits the
    budget) and advanced in groups: one group per space order, every phase
    of a step one launch over all of the group's shots (ofd_group), the
    time loop a replayed two-step graph.  A group runs until its next shot
    finishes, then is rebuilt without the finished shots; groups of the two
    space orders run on their own streams at the same time.  Retired groups
    are freed at the end, so rebuilding never waits for the device."""
    built = built if built is not None else [s.build() for s in shots]
    _last_prepare_s[0] = 0.0
    t0 = time.perf_counter()
    pending = list(enumerate(shots))
    outs = {}
    while pending:
        group, used = [], 0
        while pending:
            i, s = pending[0]
            fp = _footprint(s)
            if group and used + fp > budget_bytes:
                break
            pending.pop(0)
            group.append((i, s))
            used += fp
        tp = time.perf_counter()
        sims = {i: prepare(s, tuned=False, built=built[i]) for i, s in group}
        _last_prepare_s[0] += time.perf_counter() - tp
        rem = {i: s.steps for i, s in group}
        retired = []
        by_so = {}
        for i, s in group:
            by_so.setdefault(s.so, []).append(i)
        while any(rem.values()):
            for so, ids in by_so.items():
                live = [i for i in ids if rem[i] > 0]
                if not live:
                    continue
                k = min(rem[i] for i in live)
                for g in runtime.make_groups([sims[i] for i in live], chunk_planes=chunk_planes):
                    g.step(k)
                    retired.append(g)
                for i in live:
                    rem[i] -= k
        for g in retired:
            g.sync()
        for g in retired:
            g.close()
        for i, s in group:
            sims[i].sync()
            if keep is not None and i in keep:
                outs[i] = {f: sims[i].download(f) for f in runtime.FIELDS}
            sims[i].close()
    return time.perf_counter() - t0, outs


EDGE_CLASSES = ((32, 64), (64, 96), (96, 128), (128, 193))


def breakdown(shots, built, budget_bytes=150e9):
    """Where the batched speed-up comes from: the shots binned by grid edge
    and space order, each bin run grouped and one by one on its own.
    Returns per bin the shot count, its share of all grid-point updates and
    both arms' time and GLUP/s.  Run bin by bin, the whole workload's
    speed-up is sum(one-by-one time) / sum(grouped time); the bins holding
    most of the work bound it: with every other bin free it could not exceed
    sum(one-by-one time) / (those bins' grouped time)."""
    total = sum(s.lups for s in shots)
    out = []
    for so in sorted({s.so for s in shots}):
        for lo, hi in EDGE_CLASSES:
            idx = [i for i, s in enumerate(shots) if s.so == so and lo <= s.n < hi]
            if not idx:
                continue
            sub = [shots[i] for i in idx]
            sb = [built[i] for i in idx]
            lups = sum(s.lups for s in sub)
            tg, _ = run_grouped(sub, budget_bytes=budget_bytes, built=sb)
            to, _ = run_one_by_one(sub, built=sb)
            out.append({'space_order': so, 'edge': [lo, hi - 1], 'shots': len(sub), 'lup_share': lups / total,
                        'grouped_s': tg, 'one_by_one_s': to, 'grouped_glups': lups / tg / 1e9,
                        'one_by_one_glups': lups / to / 1e9, 'speedup': to / tg})
    return out


def _footprint(shot):
    m = shot.so // 2
    dims = (shot.n + 2 * m,) * 3
    cfg = runtime.make_config(dims, shot.so, [shot.h] * 3, 1e-3, _weights(shot.so), storage='f32')
    return runtime.Simulation.footprint(cfg)


def main():
    ap = argparse.ArgumentParser(description='batched vs one-by-one shots')
    ap.add_argument('--shots', type=int, default=256)
    ap.add_argument('--seed', type=int, default=0)
    ap.add_argument('--budget-gb', type=float, default=150.0)
    ap.add_argument('--skip-one-by-one', action='store_true')
    ap.add_argument('--chunk-planes', type=int, default=0, help='x planes per sweep CTA in groups (0: heuristic)')
    ap.add_argument('--breakdown', action='store_true',
                    help='also run every (space order, edge) bin grouped and one by one on its own')
    args = ap.parse_args()
    os.environ.setdefault('CUDA_DEVICE_MAX_CONNECTIONS', '32')
    # under torchrun: one replica per GPU, shots split round robin
    from . import replicas
    rank, world, local = replicas.rank_env()
    runtime.set_device(local)
    shots = replicas.shard(make_shots(args.shots, args.seed), rank, world)
    lups = sum(s.lups for s in shots)
    # synthesise every shot's inputs once, outside both timings
    t0 = time.perf_counter()
    built = [s.build() for s in shots]
    build_s = time.perf_counter() - t0
    # tune every distinct shape first (cached), outside both timings
    t0 = time.perf_counter()
    for b in built:
        autotune.tune(b[0], b[4], b[5], het=1)
    tune_s = time.perf_counter() - t0
    tg, _ = run_grouped(shots, budget_bytes=args.budget_gb * 1e9, built=built, chunk_planes=args.chunk_planes)
    tb, _ = run_batched(shots, budget_bytes=args.budget_gb * 1e9, built=built)
    res = {'shots': len(shots), 'glup': lups / 1e9, 'grouped_s': tg, 'grouped_glups': lups / tg / 1e9,
           'grouped_setup_s': _last_prepare_s[0],
           'streams_s': tb, 'streams_glups': lups / tb / 1e9,
           'tune_s': tune_s, 'input_synthesis_s': build_s, 'chunk_planes': args.chunk_planes,
           'edges': [s.n for s in shots], 'space_orders': [s.so for s in shots], 'steps': [s.steps for s in shots]}
    if not args.skip_one_by_one:
        to, _ = run_one_by_one(shots, built=built)
        res.update({'one_by_one_s': to, 'one_by_one_glups': lups / to / 1e9, 'speedup': to / tg,
                    'speedup_streams': to / tb})
    if args.breakdown:
        res['breakdown'] = breakdown(shots, built, budget_bytes=args.budget_gb * 1e9)
    res.update({'rank': rank, 'world': world})
    print(json.dumps(res))


if __name__ == '__main__':
    main()
