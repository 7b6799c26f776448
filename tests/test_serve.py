"""Continuous-batching server: request stream, admission under a memory
budget, and results identical alone and in the mix."""
import numpy as np
import pytest

from opesci import serve


def test_requests_are_seeded_and_rate_independent():
    a = serve.make_requests(30, 1.0, seed=4)
    b = serve.make_requests(30, 4.0, seed=4)
    assert [r.shot.n for r in a] == [r.shot.n for r in b]
    assert [r.storage for r in a] == [r.storage for r in b]
    assert np.allclose([r.arrival for r in a], [4.0 * r.arrival for r in b])
    assert all(48 <= r.shot.n <= 384 and 200 <= r.shot.steps <= 2000 for r in a)


@pytest.mark.gpu
def test_served_results_equal_alone_results():
    reqs = serve.make_requests(10, 200.0, seed=9, edge_range=(24, 56), steps_range=(20, 60), fp16_fraction=0.3)
    built = {r.id: r.shot.build() for r in reqs}
    mix, alone = {}, {}
    st = serve.serve_continuous(reqs, built, budget_bytes=2e9, slice_steps=8, checks=mix)
    serve.serve_one_by_one(reqs, built, checks=alone)
    assert serve.max_rel_diff(mix, alone) == 0.0
    assert st['p99_s'] >= st['p50_s'] > 0
    assert any(r.storage == 'f16' for r in reqs)


@pytest.mark.gpu
def test_grouped_server_results_equal_alone_results():
    """Grouped continuous batching (requests of one space order, storage and
    parity share every launch; small grids step alone) answers each request
    with the fields it gets alone."""
    reqs = serve.make_requests(14, 300.0, seed=11, edge_range=(24, 72), steps_range=(15, 70), fp16_fraction=0.3)
    built = {r.id: r.shot.build() for r in reqs}
    mix, alone = {}, {}
    st = serve.serve_grouped(reqs, built, budget_bytes=4e9, slice_steps=6, checks=mix)
    serve.serve_one_by_one(reqs, built, checks=alone)
    assert serve.max_rel_diff(mix, alone) == 0.0
    assert st['p99_s'] >= st['p50_s'] > 0
    assert any(r.storage == 'f16' for r in reqs) and any(r.shot.n < 32 for r in reqs)


@pytest.mark.gpu
def test_budget_limits_admission():
    reqs = serve.make_requests(6, 1000.0, seed=2, edge_range=(40, 48), steps_range=(20, 30), fp16_fraction=0.0)
    built = {r.id: r.shot.build() for r in reqs}
    one = serve.footprint(reqs[0])
    # a budget of about one request forces requests to run one after another
    serve.serve_continuous(reqs, built, budget_bytes=1.2 * one, slice_steps=4)
    order = sorted(reqs, key=lambda r: r.admitted)
    for a, b in zip(order, order[1:]):
        assert b.admitted >= a.finished - 1e-6 or serve.footprint(a) + serve.footprint(b) <= 1.2 * one
