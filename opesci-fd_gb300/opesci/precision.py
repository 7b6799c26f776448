"""Reduced-precision field storage: FP16 / BF16 fields with per-field
power-of-two scales, FP32 stencil arithmetic, error against an FP64 run.

Storage is value * scale rounded to the 16-bit type; the kernels multiply by
1/scale after each load and by scale before each store, so all arithmetic
stays FP32 (FP64 for the reference run).  Scales are powers of two, so the
scaling itself is exact and only the 16-bit rounding remains.

    python -m opesci.precision study --size 768 --space-order 8 --steps 800
    python -m opesci.precision convergence --sizes 64 128 256

print one JSON object each (run from opesci-fd_gb300/, or with it on
PYTHONPATH).  Storage names: f64, f32, f16, bf16, and f16sr / bf16sr for the
16-bit types with stochastic rounding of the sweeps' stores.
"""
import argparse
import json
import math
import time

import numpy as np

from . import runtime
from .models import layered_problem, eigenwave_grid, initial_fields, l2_error

FP16_MAX = 65504.0
FIELDS = runtime.FIELDS


def split_storage(name):
    """'f16sr' / 'bf16sr' -> (storage, 'stochastic'); others -> (name, 'nearest')."""
    if name.endswith('sr'):
        return name[:-2], 'stochastic'
    return name, 'nearest'


def choose_scales(absmax, storage, headroom=8.0):
    """Per-field power-of-two scales: FP16 keeps max|f| * scale within
    65504/headroom (largest such power of two); BF16, FP32 and FP64 use 1."""
    storage = split_storage(storage)[0]
    if storage not in ('f16', 'fp16', 'half'):
        return [1.0] * 9
    out = []
    for a in absmax:
        if not a > 0:
            out.append(1.0)
            continue
        k = math.floor(math.log2(FP16_MAX / headroom / a))
        out.append(float(2.0 ** max(min(k, 100), -100)))
    return out


def _problem_sim(grid, media, src, wav, storage, scales=None):
    st, rounding = split_storage(storage)
    cfg = runtime.config_from_grid(grid, storage=st, field_scale=scales, rounding=rounding)
    sim = runtime.Simulation(cfg)
    sim.set_coefficients_from_grid(grid)
    sim.set_media(*media)
    sim.set_source(src, wav)
    return sim


def precision_study(n=128, space_order=8, steps=200, seed=0, storages=('f32', 'f16', 'bf16', 'f16sr', 'bf16sr'),
                    checkpoints=8):
    """Config-3 style study on an n^3 layered problem: returns, per storage,
    the per-field relative L2 error of the final state against an FP64 run,
    with the scales used and the run times."""
    grid, media, src, wav = layered_problem(n, space_order=space_order, ntsteps=steps, seed=seed)
    out = {'grid': [n, n, n], 'space_order': space_order, 'steps': steps, 'seed': seed, 'runs': {}}
    ref = _problem_sim(grid, media, src, wav, 'f64')
    absmax = np.zeros(9)
    every = max(1, steps // checkpoints)
    t0 = time.perf_counter()
    done = 0
    while done < steps:
        k = min(every, steps - done)
        ref.step(k)
        done += k
        absmax = np.maximum(absmax, ref.absmax())
    ref.sync()
    out['runs']['f64'] = {'seconds': time.perf_counter() - t0, 'absmax': absmax.tolist()}
    for st in storages:
        scales = choose_scales(absmax, st)
        sim = _problem_sim(grid, media, src, wav, st, scales)
        t0 = time.perf_counter()
        sim.step(steps)
        sim.sync()
        secs = time.perf_counter() - t0
        errs = {}
        for f in FIELDS:
            a = sim.download(f).astype(np.float64)
            b = ref.download(f).astype(np.float64)
            errs[f] = float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
            del a, b
        sim.close()
        out['runs'][st] = {'rel_l2_vs_f64': errs, 'scales': scales, 'seconds': secs}
    ref.close()
    return out


def eigen_errors(n, storage, tmax=0.25, c=4.096, space_order=4):
    """Analytic-solution L2 errors of the eigenmode on an n^3 grid with the
    reference's refinement rule dt = c h^2 (tests/eigenwave3d.py:254-257)."""
    h = 1.0 / n
    dt = c * h * h
    steps = int(round(tmax / dt))
    g = eigenwave_grid(grid_size=(n, n, n), dt=dt, ntsteps=steps, space_order=space_order)
    A = math.sqrt(2 * g.defined_variable['mu'].value / g.defined_variable['beta'].value)
    scales = choose_scales([2.0] * 3 + [2.0 * A] * 6, storage)
    st, rounding = split_storage(storage)
    sim = runtime.Simulation(runtime.config_from_grid(g, storage=st, field_scale=scales, rounding=rounding))
    sim.set_coefficients_from_grid(g)
    dv = g.defined_variable
    sim.set_media_const(dv['beta'].value, dv['lambda'].value, dv['mu'].value)
    for k, v in initial_fields(g).items():
        sim.upload(k, 0, v)
    sim.boundary_init(0)
    sim.step(steps)
    sim.sync()
    errs = {f.label.name: l2_error(g, f, sim.download(f.label.name)) for f in g.fields}
    sim.close()
    return {'n': n, 'dt': dt, 'steps': steps, 'l2': errs}


def convergence_study(sizes=(64, 128, 256), storages=('f64', 'f32', 'f16', 'bf16', 'f16sr', 'bf16sr'), tmax=0.25,
                      c=4.096):
    """Errors and observed orders log2(e_h / e_h/2) per storage and field."""
    out = {'sizes': list(sizes), 'tmax': tmax, 'c': c, 'runs': {}}
    for st in storages:
        rows = [eigen_errors(n, st, tmax=tmax, c=c) for n in sizes]
        orders = {}
        for f in FIELDS:
            e = [r['l2'][f] for r in rows]
            orders[f] = [math.log2(e[i] / e[i + 1]) if e[i + 1] > 0 and e[i] > 0 else None
                         for i in range(len(e) - 1)]
        out['runs'][st] = {'errors': rows, 'orders': orders}
    return out


def main():
    ap = argparse.ArgumentParser(description=__doc__.split('\n')[0])
    sub = ap.add_subparsers(dest='what', required=True)
    s1 = sub.add_parser('study')
    s1.add_argument('--size', type=int, default=128)
    s1.add_argument('--space-order', type=int, default=8)
    s1.add_argument('--steps', type=int, default=200)
    s1.add_argument('--seed', type=int, default=0)
    s2 = sub.add_parser('convergence')
    s2.add_argument('--sizes', type=int, nargs='+', default=[64, 128, 256])
    s2.add_argument('--tmax', type=float, default=0.25)
    args = ap.parse_args()
    if args.what == 'study':
        res = precision_study(args.size, args.space_order, args.steps, args.seed)
    else:
        res = convergence_study(tuple(args.sizes), tmax=args.tmax)
    print(json.dumps(res))


if __name__ == '__main__':
    main()
