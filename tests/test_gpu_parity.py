"""GPU parity: the CUDA device runtime (libofd, called through its C ABI)
against the oracle, the reference-shaped C++ program run on the CPU.

Tolerance: FP32, every field within 1e-5 relative L2 of the oracle after the
run.  For the heterogeneous problem with a source every field is a
propagating wave and the norm is each field's own.  The eigenmode trades its
energy between velocities and stresses: its shear stresses are zero
analytically (their values are rounding residue of cancelling differences)
and at some final times the normal stresses are near zero too (sin(Omega t)
= 0 at t = 2 for the reference's own test3d problem).  For the eigenmode each
field's difference is therefore measured against the norm of the whole
nine-field state, the quantity the scheme conserves.
"""
import json
import os

import numpy as np
import pytest

from opesci import runtime
from opesci.models import eigenwave_grid, initial_fields, l2_error, layered_problem
from oracle import run as orun

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), 'golden')
TOL = 1e-5
SHEAR = ('Txy', 'Tyz', 'Txz')
STRESS = ('Txx', 'Tyy', 'Tzz', 'Txy', 'Tyz', 'Txz')


def run_eigen_gpu(g, variant=0, storage=None, steps=None):
    sim = runtime.Simulation(runtime.config_from_grid(g, kernel_variant=variant, storage=storage))
    sim.set_coefficients_from_grid(g)
    dv = g.defined_variable
    sim.set_media_const(dv['beta'].value, dv['lambda'].value, dv['mu'].value)
    for k, v in initial_fields(g).items():
        sim.upload(k, 0, v)
    sim.boundary_init(0)
    sim.step(steps if steps is not None else g.ntsteps.value)
    sim.sync()
    out = {f: sim.download(f) for f in runtime.FIELDS}
    sim.close()
    return out


def run_problem_gpu(g, media, src, wav, variant=0, storage='f32'):
    sim = runtime.Simulation(runtime.config_from_grid(g, kernel_variant=variant, storage=storage))
    sim.set_coefficients_from_grid(g)
    sim.set_media(*media)
    sim.set_source(src, wav)
    sim.step(g.ntsteps.value)
    sim.sync()
    out = {f: sim.download(f) for f in runtime.FIELDS}
    sim.close()
    return out


def rel_errors(got, ref, state_norm=False):
    """Per-field relative L2 differences; with state_norm the denominator is
    the norm of the whole nine-field state instead of the field's own."""
    state = np.sqrt(sum(np.linalg.norm(ref[f].astype(np.float64)) ** 2 for f in runtime.FIELDS))
    out = {}
    for f in runtime.FIELDS:
        a, b = got[f].astype(np.float64), ref[f].astype(np.float64)
        den = state if state_norm else np.linalg.norm(b)
        out[f] = float(np.linalg.norm(a - b) / max(den, 1e-300))
    return out


@pytest.mark.parametrize('so,n,steps', [(4, 32, 100), (8, 32, 60), (2, 24, 60), (6, 24, 60),
                                        # tests/eigenwave3d.py's case: 64^3 unit cube, SO4, 200 steps
                                        (4, 64, 200)])
def test_eigenwave_matches_oracle(tmp_path, so, n, steps):
    g = eigenwave_grid(grid_size=(n, n, n), ntsteps=steps, space_order=so)
    got = run_eigen_gpu(g)
    ref = orun.run(g, str(tmp_path))
    errs = rel_errors(got, ref['fields'], state_norm=True)
    assert max(errs.values()) < TOL, errs
    # analytic-solution error norms, FP64 on both sides
    for f in g.fields:
        name = f.label.name
        e_gpu = l2_error(g, f, got[name])
        assert abs(e_gpu - ref['l2_fp64'][name]) <= 1e-4 * ref['l2_fp64'][name] + 1e-12, name


@pytest.mark.parametrize('so', [2, 4, 6, 8])
def test_heterogeneous_source_matches_oracle(tmp_path, so):
    files = {k: str(tmp_path / (k + '.raw')) for k in ('rho', 'vp', 'vs')}
    g, media, src, wav = layered_problem(40, space_order=so, ntsteps=120, seed=11, media_files=files)
    got = run_problem_gpu(g, media, src, wav)
    ref = orun.run(g, str(tmp_path), source=(src, wav))
    errs = rel_errors(got, ref['fields'])
    assert max(errs.values()) < TOL, errs
    assert np.abs(got['Txx']).max() > 0
    # the sweeps evaluate the reference's own printed expression without
    # contraction; Robertsson ghosts (SO2/6/8) are exact zeros and mirrors, and
    # the SO4 Levander ghosts are the printed ghost equations (generated
    # ghost expressions): the run is bit-identical to the reference's C++
    for f in runtime.FIELDS:
        assert np.array_equal(got[f], ref['fields'][f]), f


def test_legacy_gpu_reproduces_reference_test3d(tmp_path):
    """The reference's own program benchmarks/test3d.cpp (100^3, 1000 steps):
    GPU fields against the legacy oracle, and GPU error norms against the
    norms the reference binary printed.  The reference accumulates its norms
    in float (staggeredgrid.py:916), which by itself moves them by ~1e-3
    relative from the exact sum, so that last comparison uses 2e-3."""
    gold = json.load(open(os.path.join(GOLDEN, 'test3d_l2.json')))
    g = eigenwave_grid(grid_size=(100, 100, 100), dt=0.002, ntsteps=1000, legacy=True)
    got = run_eigen_gpu(g)
    ref = orun.run(g, str(tmp_path), legacy=True)
    errs = rel_errors(got, ref['fields'], state_norm=True)
    assert max(errs.values()) < TOL, errs
    for f in g.fields:
        name = f.label.name
        e = l2_error(g, f, got[name])
        assert abs(e - ref['l2_fp64'][name]) < 1e-4 * ref['l2_fp64'][name], name
        assert abs(e - gold['l2'][name]) < 2e-3 * gold['l2'][name], (name, e, gold['l2'][name])


@pytest.mark.parametrize('so,n', [(2, 70), (4, 72), (4, 101), (6, 66)])
def test_tiled_and_plain_kernels_identical(so, n):
    """The TMA-tiled sweeps evaluate the same generated expression as the
    plain sweeps: results are bit-identical, also with partial tiles."""
    g, media, src, wav = layered_problem(n, space_order=so, ntsteps=24, seed=5)
    a = run_problem_gpu(g, media, src, wav, variant=0)
    b = run_problem_gpu(g, media, src, wav, variant=1)
    for f in runtime.FIELDS:
        assert np.array_equal(a[f], b[f]), f
    assert np.abs(a['Txx']).max() > 0


FACE_MIXES = {
    'levander': ['levander'] * 6,
    'robertsson': ['robertsson'] * 6,
    'mixed': ['levander', 'robertsson', 'robertsson', 'levander', 'robertsson', 'levander'],
    'zfree': ['none', 'none', 'none', 'none', 'levander', 'robertsson'],
}


def run_random_state(so, n, faces, storage, mode, steps=6, schedule=None):
    """Layered media, random initial fields everywhere (so every ghost and
    recompute path sees non-zero data), ``steps`` steps.  mode: 'tiled',
    'plain' (kernel variant 1) or 'persistent'.  A storage name ending in
    'sr' selects stochastic rounding of the 16-bit stores."""
    from opesci.batch import Shot
    cfg, media, src, wav, ks, kv = Shot(n, so, steps, 21, 12.0).build()
    rounding = 'stochastic' if storage.endswith('sr') else 'nearest'
    storage = storage[:-2] if storage.endswith('sr') else storage
    # velocities ~1e-7 m/s and stresses ~1 Pa, as in the layered problems
    scales = [2.0 ** 30] * 3 + [2.0 ** 9] * 6 if storage in ('f16', 'bf16') else None
    c = runtime.make_config(list(cfg.dim), so, list(cfg.spacing), cfg.dt, list(cfg.weights), storage=storage,
                            free_surface=faces, field_scale=scales, kernel_variant=1 if mode == 'plain' else 0,
                            rounding=rounding)
    sim = runtime.Simulation(c)
    sim.set_coefficients(1, ks, kv)
    sim.set_het_ghost_coefficients()
    sim.set_media(*media)
    sim.set_source(src, wav)
    rng = np.random.default_rng(so * 1000 + n)
    for f in runtime.FIELDS:
        sim.upload(f, 0, rng.standard_normal(tuple(cfg.dim)).astype(np.float32) * (1e-7 if f in 'UVW' else 1.0))
    sim.boundary_init(0)
    if schedule is not None:
        sim.set_ghost_schedule(*schedule)
    if mode == 'persistent':
        sim.set_persistent(1)
        sim.step_graph(steps)
    elif mode == 'graph':
        sim.step_graph(steps)
    else:
        sim.step(steps)
    sim.sync()
    out = {f: sim.download(f) for f in runtime.FIELDS}
    sim.close()
    return out


@pytest.mark.parametrize('so,n,faces,storage', [
    (4, 72, 'levander', 'f32'), (4, 70, 'mixed', 'f32'), (4, 66, 'zfree', 'f32'), (4, 72, 'levander', 'f16'),
    (8, 68, 'robertsson', 'f32'), (6, 67, 'mixed', 'f32'), (2, 70, 'robertsson', 'f32'),
    (8, 66, 'robertsson', 'bf16'),
    # stochastic rounding of the 16-bit stores (same hash on every path)
    (4, 72, 'levander', 'f16sr'), (8, 66, 'mixed', 'bf16sr'), (6, 67, 'robertsson', 'f16sr'),
    # four z tiles
    (4, 200, 'levander', 'f32'), (8, 196, 'mixed', 'f32'), (4, 193, 'zfree', 'f16')])
def test_boundary_paths_identical_across_kernels(so, n, faces, storage):
    """Tiled sweeps (launches and graphs), plain sweeps and persistent
    stepping agree bit for bit with every boundary active."""
    a = run_random_state(so, n, FACE_MIXES[faces], storage, 'tiled')
    b = run_random_state(so, n, FACE_MIXES[faces], storage, 'plain')
    c = run_random_state(so, n, FACE_MIXES[faces], storage, 'persistent')
    e = run_random_state(so, n, FACE_MIXES[faces], storage, 'graph')
    for f in runtime.FIELDS:
        assert np.isfinite(a[f]).all(), f
        assert np.array_equal(a[f], b[f]), ('tiled/plain', f)
        assert np.array_equal(b[f], c[f]), ('plain/persistent', f)
        assert np.array_equal(a[f], e[f]), ('steps/graph', f)


@pytest.mark.parametrize('storage', ['f32', 'f16'])
def test_ghost_schedules_identical(storage):
    """The generated space-order-4 ghosts' recompute after the stress sweep
    or beside it on the second stream, with any grid size, launched or
    replayed from graphs: bit-identical results."""
    runs = [run_random_state(4, 72, FACE_MIXES['levander'], storage, mode, schedule=sch)
            for mode, sch in (('tiled', (1, 4)), ('tiled', (0, 4)), ('graph', (0, 16)), ('graph', (1, 1)))]
    for r in runs[1:]:
        for f in runtime.FIELDS:
            assert np.array_equal(runs[0][f], r[f]), f


def test_tiled_constant_media_identical():
    g = eigenwave_grid(grid_size=(80, 80, 80), ntsteps=12, space_order=4)
    a = run_eigen_gpu(g, variant=0)
    b = run_eigen_gpu(g, variant=1)
    for f in runtime.FIELDS:
        assert np.array_equal(a[f], b[f]), f


def test_steps_are_resumable():
    """Advancing 30 steps in three calls equals one call of 30 (the
    time-slice mechanism serving relies on)."""
    g, media, src, wav = layered_problem(32, space_order=4, ntsteps=30, seed=2)
    a = run_problem_gpu(g, media, src, wav)
    sim = runtime.Simulation(runtime.config_from_grid(g))
    sim.set_coefficients_from_grid(g)
    sim.set_media(*media)
    sim.set_source(src, wav)
    for n in (7, 13, 10):
        sim.step(n)
    sim.sync()
    b = {f: sim.download(f) for f in runtime.FIELDS}
    sim.close()
    for f in runtime.FIELDS:
        assert np.array_equal(a[f], b[f]), f


def test_error_paths_leave_context_usable():
    from opesci.runtime import OFDError
    g, media, src, wav = layered_problem(24, space_order=4, ntsteps=5, seed=1)
    sim = runtime.Simulation(runtime.config_from_grid(g))
    sim.set_coefficients_from_grid(g)
    with pytest.raises(OFDError, match='outside'):
        sim.set_source((10000, 1, 1), wav)
    with pytest.raises(OFDError, match='bad field'):
        sim.download(42, 0)
    sim.set_media(*media)
    sim.step(5)
    sim.sync()
    assert np.isfinite(sim.sumsq()).all()
    sim.close()


def test_source_upload_is_ordered_while_gpu_busy():
    """A handle's inputs must be ordered with its own stream even while other
    handles keep the GPU busy (an unordered wavelet upload once let the first
    source injections read a partly copied wavelet under load)."""
    busy_g, busy_media, busy_src, busy_wav = layered_problem(160, space_order=4, ntsteps=400, seed=7)
    busy = runtime.Simulation(runtime.config_from_grid(busy_g))
    busy.set_coefficients_from_grid(busy_g)
    busy.set_media(*busy_media)
    busy.set_source(busy_src, busy_wav)
    g, media, src, wav = layered_problem(40, space_order=4, ntsteps=60, seed=8)
    alone = run_problem_gpu(g, media, src, wav)
    results = []
    for _ in range(3):
        busy.step(150)                      # keeps the device busy meanwhile
        sim = runtime.Simulation(runtime.config_from_grid(g))
        sim.set_coefficients_from_grid(g)
        sim.set_media(*media)
        sim.set_source(src, wav)
        sim.step_graph(60)
        sim.sync()
        results.append({f: sim.download(f) for f in runtime.FIELDS})
        sim.close()
    busy.sync()
    busy.close()
    for r in results:
        for f in runtime.FIELDS:
            assert np.array_equal(r[f], alone[f]), f


@pytest.mark.parametrize('so,n,storage', [(4, 40, 'f32'), (8, 36, 'f32'), (4, 33, 'f16'), (6, 30, 'f32')])
def test_persistent_steps_identical(so, n, storage):
    """Whole steps in one cooperative launch (grid barriers between phases)
    give the per-kernel results bit for bit, across launch chunks and odd
    step counts."""
    g, media, src, wav = layered_problem(n, space_order=so, ntsteps=37, seed=13)
    scales = [2.0 ** 30] * 3 + [2.0 ** 9] * 6 if storage == 'f16' else None
    out = []
    for persistent in (False, True):
        sim = runtime.Simulation(runtime.config_from_grid(g, storage=storage, field_scale=scales))
        sim.set_coefficients_from_grid(g)
        sim.set_media(*media)
        sim.set_source(src, wav)
        sim.set_persistent(persistent)
        sim.step(11)
        sim.step_graph(26)
        sim.sync()
        out.append({f: sim.download(f) for f in runtime.FIELDS})
        sim.close()
    for f in runtime.FIELDS:
        assert np.array_equal(out[0][f], out[1][f]), f
    assert np.abs(out[1]['Txx']).max() > 0


@pytest.mark.parametrize('so', [4, 8])
def test_three_source_signals_match_oracle(tmp_path, so):
    """Separate x, y and z source signals (the reference driver's xsrc, ysrc
    and zsrc, test_ref_iso_elastic.cpp:100-126,274-290) through
    ofd_set_source_xyz: bit-identical to the oracle with per-step launches,
    graph replay, persistent stepping and as a member of a group."""
    files = {k: str(tmp_path / (k + '.raw')) for k in ('rho', 'vp', 'vs')}
    g, media, src, wav = layered_problem(40, space_order=so, ntsteps=60, seed=17, media_files=files)
    w = np.asarray(wav, dtype=np.float32)
    sigs = np.stack([w, np.float32(-0.5) * w, np.float32(0.25) * np.roll(w, 7)])
    ref = orun.run(g, str(tmp_path), source=(src, tuple([float(v) for v in s] for s in sigs)))
    nt = g.ntsteps.value

    def make():
        sim = runtime.Simulation(runtime.config_from_grid(g))
        sim.set_coefficients_from_grid(g)
        sim.set_media(*media)
        sim.set_source(src, sigs)
        return sim

    runs = {}
    for mode in ('steps', 'graph', 'persistent'):
        sim = make()
        if mode == 'persistent':
            sim.set_persistent(1)
        if mode == 'steps':
            sim.step(nt)
        else:
            sim.step_graph(nt)
        sim.sync()
        runs[mode] = {f: sim.download(f) for f in runtime.FIELDS}
        sim.close()
    sims = [make(), make()]
    grp = runtime.Group(sims)
    grp.step(nt)
    grp.sync()
    runs['group'] = {f: sims[1].download(f) for f in runtime.FIELDS}
    grp.close()
    for sim in sims:
        sim.close()
    for mode, got in runs.items():
        for f in runtime.FIELDS:
            assert np.array_equal(got[f], ref['fields'][f]), (mode, f)
    # the y and z signals are not the x one: a one-signal run differs
    one = run_problem_gpu(g, media, src, wav)
    assert not np.array_equal(one['Tyy'], runs['steps']['Tyy'])


@pytest.mark.parametrize('switches', [dict(eval_const=False), dict(expand=False, eval_const=False)])
def test_switches_off_match_oracle(tmp_path, switches):
    """expand/eval_const off: the device runs the default printed form of
    the same update; the oracle prints the grid's own form (named constants
    evaluated at run time), which rounds differently.  Each field within
    1e-5 of the state norm (oracle against oracle the two forms differ by
    ~3e-7)."""
    g = eigenwave_grid(grid_size=(32, 32, 32), ntsteps=60, space_order=4, **switches)
    got = run_eigen_gpu(g)
    ref = orun.run(g, str(tmp_path))
    errs = rel_errors(got, ref['fields'], state_norm=True)
    assert max(errs.values()) < TOL, errs
    assert all(getattr(g, k) is False for k in switches)
