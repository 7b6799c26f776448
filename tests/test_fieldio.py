"""Raw field files (the reference's dump/read format), checkpoints that
resume a device-resident run bit for bit, source and receiver files and the
reference's model helpers (against what the reference's own compiled
functions gave on the fixtures in tests/golden, io.json)."""
import ctypes
import json
import os

import numpy as np
import pytest

from opesci import batch, fieldio, runtime

GOLDEN = os.path.join(os.path.dirname(__file__), 'golden')


def _io():
    with open(os.path.join(GOLDEN, 'io.json')) as fh:
        return json.load(fh)['cases']


def _f32(hexes):
    return np.array([int(h, 16) for h in hexes], dtype=np.uint32).view(np.float32)


def test_receivers_file_as_the_reference_reads_it():
    """opesci_read_receivers on edge-case lines: signs, exponents, '.5' and
    '6.', an incomplete exponent, letters, missing and extra values, lines
    of blanks, CRLF, an overflowing and a subnormal value, no final
    newline."""
    c = _io()['receivers']
    got = fieldio.read_receivers(os.path.join(GOLDEN, c['file']))
    want = _f32(c['values_hex']).reshape(-1, 3)
    assert got.shape == want.shape
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_sources_files_as_the_reference_reads_them():
    c = _io()['sources']
    xyz, sx, sy, sz = fieldio.read_sources(*[os.path.join(GOLDEN, f) for f in [c['xyz']] + c['signals']])
    assert [xyz.size, sx.size, sy.size, sz.size] == c['counts']
    assert np.array_equal(xyz.ravel().view(np.uint32), _f32(c['xyz_hex']).view(np.uint32))
    assert np.array_equal(np.concatenate([sx, sy, sz]).view(np.uint32), _f32(c['signals_hex']).view(np.uint32))


def test_lame_constants_bit_identical_to_the_reference():
    c = _io()['lame']
    mu, lam = fieldio.lame_constants(_f32(c['vp_hex']), _f32(c['vs_hex']), _f32(c['rho_hex']))
    assert np.array_equal(mu.view(np.uint32), _f32(c['mu_hex']).view(np.uint32))
    assert np.array_equal(lam.view(np.uint32), _f32(c['lam_hex']).view(np.uint32))


def test_calculate_dt_bit_identical_to_the_reference():
    for c in _io()['dt']:
        got = fieldio.calculate_dt(_f32(c['vp_hex']), c['h'])
        assert np.float32(got).view(np.uint32) == _f32([c['dt_hex']]).view(np.uint32)[0], c['h']


def test_raw_round_trip(tmp_path):
    a = np.random.default_rng(0).standard_normal((5, 6, 7)).astype(np.float32)
    fieldio.dump_field_raw(str(tmp_path / 'f'), a)
    assert (tmp_path / 'f.raw').stat().st_size == a.nbytes
    assert np.array_equal(fieldio.read_simple_binary(str(tmp_path / 'f.raw')), a.ravel())
    assert np.array_equal(fieldio.read_simple_binary_ptr(str(tmp_path / 'f.raw'), 10), a.ravel()[:10])
    with pytest.raises(ValueError):
        fieldio.read_simple_binary_ptr(str(tmp_path / 'f.raw'), a.size + 1)


@pytest.mark.gpu
@pytest.mark.parametrize('so,n', [(4, 40), (8, 36)])
def test_checkpoint_resumes_bit_for_bit(so, n, tmp_path):
    shot = batch.Shot(n, so, 30, seed=77, f0=18.0)
    built = shot.build()
    ref = batch.prepare(shot, tuned=False, built=built)
    ref.step(30)
    ref.sync()
    a = batch.prepare(shot, tuned=False, built=built)
    a.step(13)
    fieldio.checkpoint(a, str(tmp_path / 'ck'))
    a.close()
    b = batch.prepare(shot, tuned=False, built=built)
    fieldio.restore(b, str(tmp_path / 'ck'))
    assert b.steps == 13
    b.step_graph(17)
    b.sync()
    for f in runtime.FIELDS:
        assert np.array_equal(ref.download(f), b.download(f)), f
    ref.close()
    b.close()


@pytest.mark.gpu
def test_fp64_transfers_and_checkpoint_exact(tmp_path):
    """FP64 storage: double host arrays go in and come out unchanged, and a
    checkpoint of an FP64 run (written as float64) resumes bit for bit."""
    from opesci.models import layered_problem
    g, media, src, wav = layered_problem(36, space_order=4, ntsteps=24, seed=21)

    def make():
        sim = runtime.Simulation(runtime.config_from_grid(g, storage='f64'))
        sim.set_coefficients_from_grid(g)
        sim.set_media(*media)
        sim.set_source(src, wav)
        return sim

    sim = make()
    vals = np.random.default_rng(6).standard_normal(sim.dims) * (1.0 + 2.0 ** -40)
    sim.upload('Txz', 1, vals)
    back = sim.download('Txz', 1)
    assert back.dtype == np.float64 and np.array_equal(back, vals)
    sim.zero()
    sim.step(24)
    sim.sync()
    ref = {f: sim.download(f) for f in runtime.FIELDS}
    sim.close()
    a = make()
    a.step(9)
    fieldio.checkpoint(a, str(tmp_path / 'ck64'))
    a.close()
    b = make()
    fieldio.restore(b, str(tmp_path / 'ck64'))
    b.step(15)
    b.sync()
    for f in runtime.FIELDS:
        assert np.array_equal(ref[f], b.download(f)), f
    assert np.abs(ref['Txx']).max() > 0
    b.close()
    f32 = runtime.Simulation(runtime.config_from_grid(g))
    rc = f32.lib.ofd_download_field_f64(f32.h, 0, 0, back.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    assert rc == -1 and 'OFD_F64' in f32.lib.ofd_last_error().decode()
    f32.close()
