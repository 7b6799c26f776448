"""Failure handling of the continuous-batching servers, on the host only:
cancelled requests, expired deadlines and a device allocation failure at
admission.  The device runtime is replaced by fakes with the same interface
(a simulation whose work "finishes" a moment after it is queued, and groups of
them), so these run without a GPU; the failure is made on the host, and no
device state is involved."""
import time

import numpy as np
import pytest

from opesci import serve
from opesci.runtime import OFDError


class FakeSim(object):
    def __init__(self, req, hooks):
        self.req = req
        self.steps = 0
        self.busy_until = 0.0
        self.closed = False
        self.hooks = hooks

    def done(self):
        return time.perf_counter() >= self.busy_until

    def step_graph(self, k):
        self.steps += k
        self.busy_until = time.perf_counter() + 2e-3
        hook = self.hooks.get(self.req.id)
        if hook:
            hook(self)

    def sync(self):
        assert not self.closed

    def close(self):
        self.closed = True

    def sumsq(self):
        return np.array([float(self.req.id + 1)] * 9)


class FakeGroup(object):
    def __init__(self, sims):
        self.sims = sims

    def step(self, k):
        for s in self.sims:
            s.step_graph(k)

    def done(self):
        return all(s.done() for s in self.sims)

    def sync(self):
        for s in self.sims:
            s.sync()

    def close(self):
        pass


def _requests(n, gap=0.002, steps=40):
    reqs = serve.make_requests(n, 1.0, seed=5, edge_range=(24, 32), steps_range=(steps, steps), fp16_fraction=0.0)
    for i, r in enumerate(reqs):
        r.arrival = i * gap
    return reqs


def _serve(kind, reqs, opener, budget=100.0):
    built = {r.id: None for r in reqs}
    kw = dict(budget_bytes=budget, slice_steps=4, opener=opener, footprint_fn=lambda r: 1.0)
    if kind == 'grouped':
        return serve.serve_grouped(reqs, built, grouper=lambda sims: [FakeGroup(sims)], **kw)
    return serve.serve_continuous(reqs, built, **kw)


@pytest.mark.parametrize('kind', ['continuous', 'grouped'])
def test_cancelled_requests_stop_and_free_their_memory(kind):
    reqs = _requests(6)
    opened = {}

    def cancel_after_first_slice(sim):
        if sim.steps >= 4:
            sim.req.cancel()

    hooks = {2: cancel_after_first_slice}

    def opener(r, b):
        opened[r.id] = FakeSim(r, hooks)
        return opened[r.id]

    reqs[4].cancel()   # cancelled while still queued
    st = _serve(kind, reqs, opener)
    status = {r.id: r.status for r in reqs}
    assert status[4] == 'cancelled' and 4 not in opened
    assert status[2] == 'cancelled' and opened[2].closed and opened[2].steps < reqs[2].shot.steps
    assert all(status[i] == 'done' for i in (0, 1, 3, 5))
    assert all(s.closed for s in opened.values())
    assert st['done'] == 4 and st['cancelled'] == 2 and st['p50_s'] > 0


@pytest.mark.parametrize('kind', ['continuous', 'grouped'])
def test_expired_deadline_while_queued_and_while_running(kind):
    reqs = _requests(3, gap=0.0, steps=400)
    reqs[0].deadline = 0.03     # expires while running (400 steps take ~0.2 s here)
    reqs[2].deadline = 0.01     # waits behind the others (budget of two) and expires in the queue
    opened = {}

    def opener(r, b):
        opened[r.id] = FakeSim(r, {})
        return opened[r.id]

    st = _serve(kind, reqs, opener, budget=2.0)
    assert reqs[0].status == 'expired' and opened[0].steps < 400 and opened[0].closed
    assert reqs[1].status == 'done'
    assert reqs[2].status == 'expired' and 2 not in opened
    assert st['expired'] == 2 and st['done'] == 1


@pytest.mark.parametrize('kind', ['continuous', 'grouped'])
def test_allocation_failure_at_admission_fails_only_that_request(kind):
    reqs = _requests(5)

    def opener(r, b):
        if r.id == 1:
            raise OFDError('ofd_create failed (-3): cudaMalloc of 123 field bytes failed: out of memory')
        return FakeSim(r, {})

    st = _serve(kind, reqs, opener)
    assert reqs[1].status == 'failed' and 'out of memory' in reqs[1].error
    assert all(reqs[i].status == 'done' for i in (0, 2, 3, 4))
    assert st['failed'] == 1 and st['done'] == 4


def test_device_wait_expiry_fails_the_request():
    """A request whose device work reports an expired wait at sync is
    answered as failed; the others are served."""
    reqs = _requests(3)

    class Expiring(FakeSim):
        def sync(self):
            raise OFDError('ofd_sync failed (-5): a bounded device wait expired')

    def opener(r, b):
        return Expiring(r, {}) if r.id == 0 else FakeSim(r, {})

    st = _serve('continuous', reqs, opener)
    assert reqs[0].status == 'failed' and '(-5)' in reqs[0].error
    assert st['done'] == 2
