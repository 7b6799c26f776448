"""GPU parity at the benchmarked size: the 512^3 forward-modelling problem
(seeded layered heterogeneous medium, 15 Hz Ricker source in the normal
stresses, free surfaces, 10 m spacing, dt = 0.5 x the stable step, seed 0:
the inputs bench.py times), space orders 4 and 8, against the oracle program
(the reference-shaped generated C++) on the same inputs.

At this size the tiled sweeps run with 8 z tiles, 64 y tiles and several x
chunks per tile column, so the TMA ring geometry, the chunk boundaries and
the grid of several waves are all exercised, which the small parity cases do
not reach.

Every field must be bit-identical to the oracle's at both orders (the
printed update and ghost expressions evaluated in the reference's term
order and types); the 1e-5 relative L2 bound is checked first so that a
failure reports its size.  The oracle is built with vectorisation on
(-O3 -fopenmp -ffp-contract=off): elementwise loops vectorise without any
change to the IEEE operations, so its results equal the scalar build's and it
finishes in about half the time.

The full 1000-step space-order-4 run is opt-in (OFD_RUN_SLOW=1): about three
minutes of oracle time on 16 cores.
"""
import os

import numpy as np
import pytest

from opesci import runtime
from opesci.models import layered_problem
from oracle import run as orun

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _run(tmp_path, so, steps):
    files = {k: str(tmp_path / (k + '.raw')) for k in ('rho', 'vp', 'vs')}
    g, media, src, wav = layered_problem(512, space_order=so, ntsteps=steps, seed=0, media_files=files)
    sim = runtime.Simulation(runtime.config_from_grid(g))
    sim.set_coefficients_from_grid(g)
    sim.set_media(*media)
    sim.set_source(src, wav)
    sim.step(steps)
    sim.sync()
    got = {f: sim.download(f) for f in runtime.FIELDS}
    sim.close()
    del media
    ref = orun.run(g, str(tmp_path), source=(src, wav), vectorize=True)
    errs, same = {}, {}
    for f in runtime.FIELDS:
        a, b = got[f], ref['fields'][f]
        same[f] = bool(np.array_equal(a, b))
        d = np.linalg.norm((a.astype(np.float64) - b.astype(np.float64)).ravel())
        errs[f] = float(d / max(np.linalg.norm(b.astype(np.float64).ravel()), 1e-300))
        got[f] = None
        ref['fields'][f] = None
    return errs, same


@pytest.mark.parametrize('so', [4, 8])
def test_512_heterogeneous_source_matches_oracle(tmp_path, so):
    errs, same = _run(tmp_path, so, 100)
    print('512^3 SO%d, 100 steps: relative L2 vs oracle' % so, {k: '%.2e' % v for k, v in errs.items()},
          'bit-identical fields:', [k for k, v in same.items() if v])
    assert max(errs.values()) < TOL, errs
    assert all(same.values()), same


@pytest.mark.skipif(os.environ.get('OFD_RUN_SLOW') != '1', reason='opt-in: OFD_RUN_SLOW=1 (full 1000-step run)')
def test_512_so4_full_run_matches_oracle(tmp_path):
    errs, same = _run(tmp_path, 4, 1000)
    print('512^3 SO4, 1000 steps: relative L2 vs oracle', {k: '%.2e' % v for k, v in errs.items()})
    assert max(errs.values()) < TOL, errs
    assert all(same.values()), same
