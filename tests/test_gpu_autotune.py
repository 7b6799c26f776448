"""The autotuner (opesci.autotune): it times each knob on a scratch handle of
the configuration's shape and returns the fastest; results do not depend on
the knobs, so a tuned simulation equals an untuned one bit for bit."""
import numpy as np
import pytest

from opesci import autotune, runtime
from opesci.batch import Shot

pytestmark = pytest.mark.gpu


def _run(built, knobs, steps):
    cfg, media, src, wav, ks, kv = built
    sim = runtime.Simulation(cfg)
    sim.set_coefficients(1, ks, kv)
    sim.set_het_ghost_coefficients()
    sim.set_media(*media)
    sim.set_source(src, wav)
    if knobs is not None:
        sim.set_tuning(**knobs)
    sim.step_graph(steps)
    sim.sync()
    out = {f: sim.download(f) for f in runtime.FIELDS}
    sim.close()
    return out


@pytest.mark.parametrize('so', [4, 8])
def test_tuned_knobs_leave_results_unchanged(tmp_path, monkeypatch, so):
    monkeypatch.setenv('OFD_TUNE_CACHE', str(tmp_path / 'tune.json'))
    built = Shot(72, so, 12, 3, 15.0).build()
    cfg, _, _, _, ks, kv = built
    knobs = autotune.tune(cfg, ks, kv, het=1, steps=6, use_cache=True)
    for k in autotune.DEFAULT:
        assert k in knobs
    if so == 4 and not knobs['persistent']:
        # generated ghosts: the recompute schedule was among the candidates
        cands = autotune._load()[autotune._key(cfg, 1)]['candidates']
        assert any('rc_mode' in c[0] for c in cands)
    a = _run(built, None, 12)
    b = _run(built, knobs, 12)
    for f in runtime.FIELDS:
        assert np.array_equal(a[f], b[f]), f
