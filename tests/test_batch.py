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
def test_grouped_equals_one_by_one():
    """Grouped launches (one launch per phase over all shots of a space
    order, groups rebuilt as shots finish, odd remainders) reproduce each
    shot alone bit for bit."""
    shots = [batch.Shot(n, so, st, seed=i, f0=10.0 + i) for i, (n, so, st) in
             enumerate([(33, 4, 31), (48, 8, 20), (40, 4, 17), (70, 4, 12), (36, 8, 25), (64, 8, 9),
                        (100, 4, 14), (57, 4, 31)])]
    keep = set(range(len(shots)))
    built = [s.build() for s in shots]
    _, a = batch.run_one_by_one(shots, keep=keep, built=built)
    for chunk in (0, 24):
        _, b = batch.run_grouped(shots, keep=keep, built=built, chunk_planes=chunk)
        for i in keep:
            for f in runtime.FIELDS:
                assert np.array_equal(a[i][f], b[i][f]), (chunk, i, f)


@pytest.mark.gpu
def test_group_of_16bit_members_and_member_streams():
    """A group of scaled-FP16 members, with work queued on a member's own
    stream before and after the group step, equals stepping alone."""
    scales = [2.0 ** 30] * 3 + [2.0 ** 9] * 6
    shots = [batch.Shot(n, 4, 14, seed=30 + i, f0=12.0) for i, n in enumerate((40, 52, 45))]

    def make(s):
        cfg, media, src, wav, ks, kv = s.build()
        c = runtime.make_config(list(cfg.dim), 4, list(cfg.spacing), cfg.dt, list(cfg.weights), storage='f16',
                                free_surface=list(cfg.free_surface), field_scale=scales)
        sim = runtime.Simulation(c)
        sim.set_coefficients(1, ks, kv)
        sim.set_het_ghost_coefficients()
        sim.set_media(*media)
        sim.set_source(src, wav)
        return sim

    alone = []
    for s in shots:
        sim = make(s)
        sim.step(14)
        sim.sync()
        alone.append({f: sim.download(f) for f in runtime.FIELDS})
        sim.close()
    sims = [make(s) for s in shots]
    sims[0].step(3)
    for sim in sims[1:]:
        sim.step_graph(3)
    g = runtime.Group(sims)
    g.step(9)
    sims[1].step(2)          # queued on a member stream after the group
    g.sync()
    sims[0].step(2)
    sims[2].step_graph(2)
    for i, sim in enumerate(sims):
        sim.sync()
        assert sim.steps == 14
        for f in runtime.FIELDS:
            assert np.array_equal(alone[i][f], sim.download(f)), (i, f)
    g.close()
    for sim in sims:
        sim.close()


@pytest.mark.gpu
def test_group_rejects_unfit_members():
    a = batch.prepare(batch.Shot(40, 4, 5, seed=1, f0=10.0), tuned=False)
    b = batch.prepare(batch.Shot(40, 8, 5, seed=2, f0=10.0), tuned=False)
    c = batch.prepare(batch.Shot(40, 4, 5, seed=3, f0=10.0), tuned=False)
    tiny = batch.prepare(batch.Shot(12, 4, 5, seed=4, f0=10.0), tuned=False)
    c.step(1)
    for members, msg in (([a, b], 'space order'), ([a, c], 'time level'), ([a, tiny], 'tiled'),
                         ([a, a], 'twice')):
        with pytest.raises(runtime.OFDError, match=msg):
            runtime.Group(members)
    for x in (a, b, c, tiny):
        x.close()


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
