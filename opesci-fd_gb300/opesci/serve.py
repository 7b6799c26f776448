"""Serving forward-modelling requests with continuous batching on one GPU.

Requests (grid edge log-uniform in [48, 384], space order 4 or 8, 200-2000
steps, FP32 or scaled-FP16 storage, seeded layered media and Ricker source)
arrive as a Poisson stream.  The server admits a waiting request as soon as
its device footprint fits the HBM budget (150 GB by default), keeps its nine
fields and media resident, and advances every admitted request in slices of
time steps.  Two forms:

* serve_grouped: each round, the requests of one space order, storage and
  time-level parity form a group (ofd_group) whose every phase is one
  launch over all of them;
* serve_continuous: each request replays its own captured graph on its own
  stream.

Requests that arrive while others run join at the next slice boundary, their
work overlaps on the device, and a finished request frees its memory for the
queue.  The baseline serves the same stream one request at a time with
per-kernel launches.

Failures are contained per request.  A request may be cancelled
(Request.cancel(), from any thread) or carry a deadline (seconds after its
arrival); a queued one is dropped, an admitted one is stopped at its next
slice boundary (after its last launched work has completed) and its memory
returns to the budget.  A request whose device state cannot be created at
admission (an allocation failure or any other error of the runtime) is
answered as failed with the error text, and serving goes on.  Each request
ends with status 'done', 'cancelled', 'expired' or 'failed'; latency and
throughput figures count the 'done' ones.

    python -m opesci.serve --requests 40 --rates 0.5 1 2

prints a JSON object: per rate, p50/p99 latency and aggregate GLUP/s for both
servers, and the largest difference between a request's result served in the
mix and served alone (FP64 sums of squares of its nine final fields).
"""
import argparse
import json
import math
import os
import time
from collections import deque

import numpy as np

from . import runtime, autotune
from .batch import Shot, _weights

# Fixed FP16 storage scales for these layered problems (unit Ricker source):
# velocities ~1e-7 m/s, stresses ~1 Pa, from the precision study's magnitudes
# with 16x headroom.
FP16_SCALES = [2.0 ** 30] * 3 + [2.0 ** 9] * 3 + [2.0 ** 10] * 3


class Request(object):
    def __init__(self, rid, arrival, shot, storage, deadline=None):
        self.id, self.arrival, self.shot, self.storage = rid, arrival, shot, storage
        self.deadline = deadline          # seconds after arrival, or None
        self.admitted = self.finished = None
        self.status = None                # 'done', 'cancelled', 'expired', 'failed'
        self.error = None
        self.cancelled = False

    @property
    def lups(self):
        return self.shot.lups

    def cancel(self):
        """Ask the server to drop this request (safe from another thread)."""
        self.cancelled = True

    def stop_reason(self, now):
        """'cancelled' / 'expired' when the request should stop at ``now``
        (server clock), else None."""
        if self.cancelled:
            return 'cancelled'
        if self.deadline is not None and now > self.arrival + self.deadline:
            return 'expired'
        return None


def make_requests(count, rate, seed=0, edge_range=(48, 384), so_choices=(4, 8), steps_range=(200, 2000),
                  fp16_fraction=0.25, f_range=(8.0, 25.0)):
    """Seeded requests; the jobs depend on ``seed`` only and the Poisson
    arrival times (mean gap 1/rate) on a second stream, so a rate sweep
    serves the same jobs at different loads."""
    rng = np.random.default_rng(seed)
    arr = np.random.default_rng(seed + 1)
    t = 0.0
    out = []
    for i in range(count):
        t += arr.exponential(1.0) / rate
        n = int(round(math.exp(rng.uniform(math.log(edge_range[0]), math.log(edge_range[1])))))
        so = int(rng.choice(so_choices))
        steps = int(rng.integers(steps_range[0], steps_range[1] + 1))
        f0 = float(rng.uniform(*f_range))
        storage = 'f16' if rng.uniform() < fp16_fraction else 'f32'
        out.append(Request(i, t, Shot(n, so, steps, seed * 7777 + i, f0), storage))
    return out


def footprint(req):
    m = req.shot.so // 2
    dims = (req.shot.n + 2 * m,) * 3
    cfg = runtime.make_config(dims, req.shot.so, [10.0] * 3, 1e-3, _weights(req.shot.so), storage=req.storage)
    return runtime.Simulation.footprint(cfg)


def open_request(req, built, tuned=True):
    cfg, media, src, wav, ks, kv = built
    scales = FP16_SCALES if req.storage == 'f16' else None
    c = runtime.make_config(list(cfg.dim), cfg.space_order, list(cfg.spacing), cfg.dt, list(cfg.weights),
                            storage=req.storage, free_surface=list(cfg.free_surface), field_scale=scales)
    sim = runtime.Simulation(c)
    sim.set_coefficients(1, ks, kv)
    sim.set_het_ghost_coefficients()
    sim.set_media(*media)
    sim.set_source(src, wav)
    if tuned and req.storage == 'f32':
        sim.set_tuning(**autotune.tune(c, ks, kv, het=1))
    return sim


def _finish_stats(reqs, t_first=None, t_last=None):
    done = [r for r in reqs if r.status == 'done']
    counts = {k: sum(1 for r in reqs if r.status == k) for k in ('done', 'cancelled', 'expired', 'failed')}
    if not done:
        return dict(counts, p50_s=None, p99_s=None, mean_s=None, glups=0.0, makespan_s=None)
    t_first = min(r.arrival for r in reqs) if t_first is None else t_first
    t_last = max(r.finished for r in reqs if r.finished is not None) if t_last is None else t_last
    lat = np.array([r.finished - r.arrival for r in done])
    lups = sum(r.lups for r in done)
    return dict(counts, p50_s=float(np.percentile(lat, 50)), p99_s=float(np.percentile(lat, 99)),
                mean_s=float(lat.mean()), glups=lups / max(t_last - t_first, 1e-12) / 1e9,
                makespan_s=t_last - t_first)


def _end(req, status, now, error=None):
    req.status, req.finished = status, now
    if error is not None:
        req.error = error


def _admit(queue, active, used, budget_bytes, max_active, now, opener, built, footprint_fn, extra):
    """Move queued requests into ``active`` while the budget allows; drops
    cancelled/expired ones and answers requests whose device state cannot be
    created as failed.  Returns the new byte count in use."""
    while queue and len(active) < max_active:
        r = queue[0]
        why = r.stop_reason(now)
        if why:
            queue.popleft()
            _end(r, why, now)
            continue
        fp = footprint_fn(r)
        if active and used + fp > budget_bytes:
            break
        queue.popleft()
        r.admitted = now
        try:
            sim = opener(r, built[r.id])
        except Exception as e:   # the request fails, the server goes on
            _end(r, 'failed', now, '%s: %s' % (type(e).__name__, e))
            continue
        active.append([r, sim, r.shot.steps, fp] + list(extra))
        used += fp
    return used


def serve_continuous(reqs, built, budget_bytes=150e9, slice_steps=32, max_active=96, checks=None,
                     opener=None, footprint_fn=footprint):
    """Continuous batching.  ``checks`` (dict) receives each request's FP64
    sums of squares of its final fields.  ``opener(req, built)`` creates a
    request's device state (default: open_request with autotuned launch
    knobs)."""
    opener = opener or open_request
    t0 = time.perf_counter()
    pending = deque(sorted(reqs, key=lambda r: r.arrival))
    queue = deque()
    active = []          # [req, sim, remaining, bytes]
    used = 0
    while pending or queue or active:
        now = time.perf_counter() - t0
        while pending and pending[0].arrival <= now:
            queue.append(pending.popleft())
        used = _admit(queue, active, used, budget_bytes, max_active, now, opener, built, footprint_fn, ())
        if not active:
            if pending:
                time.sleep(max(0.0, pending[0].arrival - (time.perf_counter() - t0)))
            elif queue:
                time.sleep(50e-6)
            continue
        progressed = False
        for a in list(active):
            r, sim, rem, fp = a
            if sim.done():
                now = time.perf_counter() - t0
                why = r.stop_reason(now) if rem > 0 else None
                if rem == 0 or why:
                    try:
                        sim.sync()          # raises if a device wait of the request expired
                        if why:
                            _end(r, why, now)
                        else:
                            _end(r, 'done', time.perf_counter() - t0)
                            if checks is not None:
                                checks[r.id] = sim.sumsq().tolist()
                    except Exception as e:
                        _end(r, 'failed', time.perf_counter() - t0, '%s: %s' % (type(e).__name__, e))
                    sim.close()
                    used -= fp
                    active.remove(a)
                else:
                    # keep two slices in flight per request
                    k = min(2 * slice_steps, rem)
                    sim.step_graph(k)
                    a[2] = rem - k
                progressed = True
        if not progressed:
            time.sleep(50e-6)
    return _finish_stats(reqs)


def serve_grouped(reqs, built, budget_bytes=150e9, slice_steps=32, max_active=256, checks=None,
                  opener=None, footprint_fn=footprint, grouper=None):
    """Continuous batching on groups.  Admission as in serve_continuous; the
    admitted requests advance in rounds: each round groups the requests
    that still have steps to run by space order, storage and time-level
    parity (ofd_group: every phase of a step one launch over the whole
    group) and advances every group by min(slice_steps, its smallest
    remaining count) steps.  Up to two rounds are in flight; a request
    that arrives joins the next round, one that finishes is answered and
    freed when its last round has completed.  A cancelled or expired
    request joins no further round and is freed when its last round has
    completed.  ``opener`` and ``grouper`` (sims -> groups) default to the
    device runtime's."""
    opener = opener or (lambda r, b: open_request(r, b, tuned=False))
    grouper = grouper or runtime.make_groups
    t0 = time.perf_counter()
    pending = deque(sorted(reqs, key=lambda r: r.arrival))
    queue = deque()
    active = []          # [req, sim, remaining, bytes, last_round]
    rounds = deque()     # (round id, [groups])
    used = 0
    next_round = 0
    completed = -1       # newest round known to have finished
    while pending or queue or active:
        now = time.perf_counter() - t0
        while pending and pending[0].arrival <= now:
            queue.append(pending.popleft())
        used = _admit(queue, active, used, budget_bytes, max_active, now, opener, built, footprint_fn, (-1,))
        # retire rounds that have finished (oldest first)
        while rounds and all(g.done() for g in rounds[0][1]):
            rid, groups = rounds.popleft()
            failed = None
            for g in groups:
                try:
                    g.sync()
                except Exception as e:   # a member's device wait expired
                    failed = '%s: %s' % (type(e).__name__, e)
                g.close()
            if failed:
                for a in active:
                    if a[4] == rid:
                        a[0].error = failed
            completed = rid
        # answer requests whose last round has completed; stop cancelled or
        # expired ones there
        now = time.perf_counter() - t0
        for a in list(active):
            r, sim, rem, fp, last = a
            why = r.stop_reason(now) if rem > 0 else None
            if (rem == 0 or why) and last <= completed:
                try:
                    sim.sync()
                    if r.error:
                        raise RuntimeError(r.error)
                    if why:
                        _end(r, why, now)
                    else:
                        _end(r, 'done', time.perf_counter() - t0)
                        if checks is not None:
                            checks[r.id] = sim.sumsq().tolist()
                except Exception as e:
                    _end(r, 'failed', time.perf_counter() - t0, '%s: %s' % (type(e).__name__, e))
                sim.close()
                used -= fp
                active.remove(a)
        live = [a for a in active if a[2] > 0 and not a[0].stop_reason(now)]
        if live and len(rounds) < 2:
            classes = {}
            for a in live:
                key = (a[0].shot.so, a[0].storage, a[1].steps % 2)
                classes.setdefault(key, []).append(a)
            groups = []
            for members in classes.values():
                k = min(slice_steps, min(a[2] for a in members))
                for g in grouper([a[1] for a in members]):
                    g.step(k)
                    groups.append(g)
                for a in members:
                    a[2] -= k
                    a[4] = next_round
            rounds.append((next_round, groups))
            next_round += 1
            continue
        if not active and not queue and pending:
            time.sleep(max(0.0, pending[0].arrival - (time.perf_counter() - t0)))
        else:
            time.sleep(50e-6)
    return _finish_stats(reqs)


def serve_one_by_one(reqs, built, checks=None):
    """Baseline: one request at a time in arrival order, per-kernel launches."""
    t0 = time.perf_counter()
    for r in sorted(reqs, key=lambda r: r.arrival):
        now = time.perf_counter() - t0
        if r.arrival > now:
            time.sleep(r.arrival - now)
        r.admitted = time.perf_counter() - t0
        sim = open_request(r, built[r.id], tuned=False)
        sim.step(r.shot.steps)
        sim.sync()
        _end(r, 'done', time.perf_counter() - t0)
        if checks is not None:
            checks[r.id] = sim.sumsq().tolist()
        sim.close()
    return _finish_stats(reqs)


def max_rel_diff(a, b):
    worst = 0.0
    for k in a:
        x, y = np.array(a[k]), np.array(b[k])
        d = np.abs(x - y) / np.maximum(np.abs(y), 1e-300)
        worst = max(worst, float(d.max()))
    return worst


def main():
    ap = argparse.ArgumentParser(description='continuous-batching server vs one request at a time')
    ap.add_argument('--requests', type=int, default=40)
    ap.add_argument('--rates', type=float, nargs='+', default=[0.5, 1.0, 2.0])
    ap.add_argument('--seed', type=int, default=0)
    ap.add_argument('--budget-gb', type=float, default=150.0)
    ap.add_argument('--max-edge', type=int, default=384)
    args = ap.parse_args()
    os.environ.setdefault('CUDA_DEVICE_MAX_CONNECTIONS', '32')
    out = {'requests': args.requests, 'rates': {}}
    jobs = make_requests(args.requests, 1.0, seed=args.seed, edge_range=(48, args.max_edge))
    built = {r.id: r.shot.build() for r in jobs}
    for r in jobs:
        if r.storage == 'f32':
            b = built[r.id]
            autotune.tune(b[0], b[4], b[5], het=1)
    out['jobs'] = [dict(r.shot.to_dict(), storage=r.storage) for r in jobs]
    for rate in args.rates:
        reqs = make_requests(args.requests, rate, seed=args.seed, edge_range=(48, args.max_edge))
        chk_g, chk_c, chk_p = {}, {}, {}
        grp = serve_grouped(reqs, built, budget_bytes=args.budget_gb * 1e9, checks=chk_g)
        reqs = make_requests(args.requests, rate, seed=args.seed, edge_range=(48, args.max_edge))
        cont = serve_continuous(reqs, built, budget_bytes=args.budget_gb * 1e9, checks=chk_c)
        reqs = make_requests(args.requests, rate, seed=args.seed, edge_range=(48, args.max_edge))
        plain = serve_one_by_one(reqs, built, checks=chk_p)
        out['rates'][str(rate)] = {
            'grouped': grp, 'continuous_streams': cont, 'one_by_one': plain,
            'glups_ratio': grp['glups'] / plain['glups'],
            'glups_ratio_streams': cont['glups'] / plain['glups'],
            'max_rel_diff_alone_vs_mix': max(max_rel_diff(chk_g, chk_p), max_rel_diff(chk_c, chk_p)),
            'fp16_requests': sum(1 for r in reqs if r.storage == 'f16'),
            'glup': sum(r.lups for r in reqs) / 1e9}
    print(json.dumps(out))


if __name__ == '__main__':
    main()
