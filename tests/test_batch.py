"""Batched shots: host-side construction (CPU) and GPU equivalence of batched
and one-by-one execution."""
import numpy as np
import pytest

from opesci import batch, runtime
from opesci.models import layered_problem
from opesci.templates import cuda_gen


def test_shot_build_matches_symbolic_problem():
    s = batch.Shot(28, 8, 40, seed=17, f0=12.5)
    cfg, media, src, wav, ks, kv = s.build()
    g, media2, src2, wav2 = layered_problem(28, space_order=8, ntsteps=40, seed=17, f0=12.5)
    ref = cuda_gen.sweep_tables(g)
    assert np.array_equal(ks, ref['stress'][1]) and np.array_equal(kv, ref['velocity'][1])
    assert src == src2 and np.array_equal(wav, wav2)
    for a, b in zip(media, media2):
        assert np.array_equal(a, b)
    gcfg = runtime.config_from_grid(g)
    assert list(cfg.dim) == list(gcfg.dim) and cfg.dt == gcfg.dt
    assert list(cfg.free_surface) == list(gcfg.free_surface)


def test_make_shots_distribution():
    shots = batch.make_shots(256, seed=0)
    edges = np.array([s.n for s in shots])
    assert edges.min() >= 32 and edges.max() <= 192
    assert set(s.so for s in shots) == {4, 8}
    assert all(300 <= s.steps <= 1500 for s in shots)
    assert all(8.0 <= s.f0 <= 25.0 for s in shots)
    # log-uniform: the median edge sits near the geometric mean of 32 and 192
    assert 60 < np.median(edges) < 100


@pytest.mark.gpu
def test_batched_equals_one_by_one():
    shots = [batch.Shot(n, so, st, seed=i, f0=10.0 + i) for i, (n, so, st) in
             enumerate([(33, 4, 31), (48, 8, 20), (40, 4, 17), (70, 4, 12), (36, 8, 25), (64, 8, 9)])]
    keep = set(range(len(shots)))
    built = [s.build() for s in shots]
    _, a = batch.run_one_by_one(shots, keep=keep, built=built)
    _, b = batch.run_batched(shots, keep=keep, built=built)
    for i in keep:
        for f in runtime.FIELDS:
            assert np.array_equal(a[i][f], b[i][f]), (i, f)


@pytest.mark.gpu
def test_graph_steps_equal_plain_steps():
    s = batch.Shot(45, 4, 23, seed=5, f0=15.0)
    built = s.build()
    x = batch.prepare(s, tuned=False, built=built)
    x.step(23)
    x.sync()
    y = batch.prepare(s, tuned=True, built=built)
    y.step_graph(10)
    y.step_graph(13)
    y.sync()
    for f in runtime.FIELDS:
        assert np.array_equal(x.download(f), y.download(f)), f
    x.close()
    y.close()
