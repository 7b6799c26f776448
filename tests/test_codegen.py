"""Generated device expressions (csrc/generated) against the frontend, on CPU.

* The sweeps' expressions read every array either at an x offset or with a
  y/z neighbour, never both: the tiled sweeps of space order >= 6 stage the x
  window as point boxes and only the current plane with y/z halos.
* The space-order-4 Levander ghost expressions printed from the frontend have
  the structure of the prebuilt header (signature), and the fast literal table
  of heterogeneous models (monomials in dt and h) equals the table the
  frontend prints for a layered model.
"""
import os
import re

import numpy as np

from opesci.models import layered_problem
from opesci.templates import cuda_gen

GEN = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), 'opesci-fd_gb300', 'csrc',
                   'generated')


def test_sweep_expressions_mix_no_offsets():
    text = open(os.path.join(GEN, 'sweeps_gen.cuh')).read()
    refs = re.findall(r'A\((F_\w+), (-?\d), (-?\d), (-?\d)\)', text)
    assert refs
    for f, dx, dy, dz in refs:
        assert sum(1 for v in (dx, dy, dz) if v != '0') <= 1, (f, dx, dy, dz)


def test_ghost_header_matches_frontend():
    sigs = cuda_gen.prebuilt_signatures()
    for het in (0, 1):
        g = cuda_gen._ghost_variant_grid(het)
        cases, lits = cuda_gen.ghost_text(g)
        key = 'so4_%s' % ('het' if het else 'const')
        assert cuda_gen.ghost_signature(cases) == sigs[key]['ghost']
        assert len(lits) == sigs[key]['nk_ghost']
    text = open(os.path.join(GEN, 'ghosts_gen.cuh')).read()
    assert len(re.findall(r'^\s+case \d+: return', text, re.M)) == 60
    # the reference's pow(mu, 2) survives as the exact double square
    assert 'ofd_pow2(A.m(M_MU, 0, 0, 0))' in text


def test_het_ghost_table_equals_frontend_table(tmp_path):
    files = {k: str(tmp_path / (k + '.raw')) for k in ('rho', 'vp', 'vs')}
    g, media, src, wav = layered_problem(20, space_order=4, ntsteps=3, seed=2, media_files=files)
    sig, tab = cuda_gen.ghost_table(g)
    assert sig == cuda_gen.prebuilt_signatures()['so4_het']['ghost']
    fast = cuda_gen.het_ghost_table(g.dt.value, g.spacing[0].value)
    assert fast.dtype == np.float32 and len(fast) == len(tab)
    assert np.array_equal(fast.view(np.uint32), tab.view(np.uint32))
