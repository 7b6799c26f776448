"""Sources and receivers: the reference's trace resampling (against its own
compiled output, tests/golden/resample.json), receiver positions, and GPU
seismograms against the oracle's."""
import json
import os

import numpy as np
import pytest

from opesci import runtime, traces, batch
from opesci.models import layered_problem
from oracle import run as orun

GOLDEN = os.path.join(os.path.dirname(__file__), 'golden')


def test_resample_matches_reference_output():
    gold = json.load(open(os.path.join(GOLDEN, 'resample.json')))
    assert len(gold['cases']) >= 5
    for c in gold['cases']:
        got = traces.resample_timeseries(np.array(c['src'], dtype=np.float32), c['dt'], c['sdt'])
        want = np.array(c['resampled'], dtype=np.float32)
        assert got.shape == want.shape, (c['dt'], c['sdt'])
        assert np.array_equal(got, want), (c['dt'], c['sdt'], float(np.abs(got - want).max()))


def test_resample_keeps_band_limited_signal():
    # a band-limited periodic signal resampled to half the interval keeps its
    # shape at the common times; the reference normalises the forward and the
    # inverse transform by 1/sqrt of their own lengths, so the amplitude
    # scales by sqrt(n / n2)
    n, sdt, dt = 128, 1e-3, 0.5e-3
    t = np.arange(n) * sdt
    s = np.sin(2 * np.pi * 5 * t / (n * sdt)).astype(np.float32)
    r = traces.resample_timeseries(s, dt, sdt)
    assert len(r) == 2 * n
    assert np.abs(r[::2] - s * np.sqrt(0.5)).max() < 1e-4


def test_receiver_indices():
    idx = traces.receiver_indices([[0.0, 10.0, 24.9], [15.0, 5.1, 4.9]], 10.0, 2)
    assert idx.tolist() == [[2, 3, 4], [4, 3, 2]]


def test_point_indices_match_reference_rounding():
    """Point indices equal the reference driver's (int)round(coor/h) (float
    quotient, half away from zero) on coordinates at and beside half-way
    ties, where a double quotient or round-half-even gives other indices."""
    gold = json.load(open(os.path.join(GOLDEN, 'io.json')))['cases']['indices']
    for case in gold:
        coor = np.array([int(x, 16) for x in case['coor_hex']], dtype=np.uint32).view(np.float32)
        want = np.array(case['index'])
        got = traces.point_indices(np.stack([coor, coor[::-1], coor], axis=1), case['h'])
        assert np.array_equal(got[:, 0], want), case['h']
        assert np.array_equal(got[:, 1], want[::-1]), case['h']
        assert np.array_equal(traces.point_indices(np.stack([coor] * 3, axis=1), case['h'], margin=4)[:, 2],
                              want + 4)
        # the planted ties separate it from a plain double-precision rounding
        assert (np.round(coor.astype(np.float64) / case['h']).astype(np.int64) != want).any(), case['h']


def _receivers(g):
    m = g.order[1] // 2
    n = [d.value for d in g.dim]
    return [(m + 3, n[1] // 2, n[2] // 2), (n[0] // 2, m + 1, m), (n[0] - m - 2, n[1] - m - 1, n[2] - m - 3),
            (n[0] // 2 + 1, n[1] // 2 - 2, n[2] // 2 + 1)]


def _problem(tmp_path, n, so, steps, seed):
    files = {k: str(tmp_path / (k + '.raw')) for k in ('rho', 'vp', 'vs')}
    return layered_problem(n, space_order=so, ntsteps=steps, seed=seed, media_files=files)


def test_oracle_records_traces(tmp_path):
    g, media, src, wav = _problem(tmp_path, 18, 4, 12, 3)
    rec = _receivers(g) + [tuple(src)]
    out = orun.run(g, str(tmp_path), source=(src, wav), receivers=rec)
    tr = out['traces']
    assert tr.shape == (12, 4, len(rec))
    assert np.abs(tr[:, 3, -1]).max() > 0          # pressure at the source point
    x, y, z = rec[0]
    assert tr[-1, 0, 0] == out['fields']['U'][x, y, z]


def _gpu_traces(g, media, src, wav, rec, mode):
    cfg = runtime.config_from_grid(g, kernel_variant=1 if mode == 'plain' else 0)
    sim = runtime.Simulation(cfg)
    sim.set_coefficients_from_grid(g)
    sim.set_media(*media)
    sim.set_source(src, wav)
    sim.set_receivers(rec, g.ntsteps.value + 3)
    n = g.ntsteps.value
    if mode == 'persistent':
        sim.set_persistent(1)
        sim.step_graph(n)
    elif mode == 'graph':
        sim.step_graph(n)
    elif mode == 'group':
        grp = runtime.Group([sim])
        grp.step(n)
        grp.sync()
        grp.close()
    else:
        sim.step(n)
    sim.sync()
    tr = sim.traces()
    sim.close()
    return tr


@pytest.mark.gpu
@pytest.mark.parametrize('so,n', [(8, 40), (4, 44)])
def test_gpu_traces_match_oracle(so, n, tmp_path):
    """Seismograms (U, V, W, P at receivers, every step) recorded on the GPU
    equal the oracle's bit for bit, at space order 8 (Robertsson ghosts) and
    at space order 4 (the generated Levander ghosts), in every stepping
    path."""
    g, media, src, wav = _problem(tmp_path, n, so, 30, 6)
    rec = _receivers(g) + [tuple(src)]
    ref = orun.run(g, str(tmp_path), source=(src, wav), receivers=rec)['traces']
    for mode in ('step', 'graph', 'persistent', 'group', 'plain'):
        tr = _gpu_traces(g, media, src, wav, rec, mode)
        assert tr.shape == (33, 4, len(rec))
        assert not tr[30:].any()                    # rows beyond the steps run stay zero
        got = tr[:30]
        peak = np.maximum(np.abs(ref).max(axis=0), 1e-30)
        assert np.array_equal(got, ref), (mode, float((np.abs(got - ref).max(axis=0) / peak).max()))
    assert np.abs(ref[:, 3, -1]).max() > 0


@pytest.mark.gpu
def test_group_members_keep_their_receivers():
    shots = [batch.Shot(n, 4, 16, seed=40 + i, f0=14.0) for i, n in enumerate((36, 44))]
    alone, sims = [], []
    for s in shots:
        for keep in (alone, sims):
            sim = batch.prepare(s, tuned=False)
            m = 2
            sim.set_receivers([(m + 5, m + 6, m + 7), (m + 9, m + 3, m + 11)], 16)
            keep.append(sim)
    for sim in alone:
        sim.step(16)
        sim.sync()
    g = runtime.Group(sims)
    g.step(16)
    g.sync()
    g.close()
    for a, b in zip(alone, sims):
        assert np.array_equal(a.traces(), b.traces())
        a.close()
        b.close()
