"""SEG-Y earth models: header parsing and IBM-float decoding against what the
reference's own opesci_read_model_segy reads from the same files
(tests/golden/segy.json), on the host and on the GPU."""
import json
import os

import numpy as np
import pytest

from opesci import segy

GOLDEN = os.path.join(os.path.dirname(__file__), 'golden')


def _gold():
    return json.load(open(os.path.join(GOLDEN, 'segy.json')))['files']


def _bits(a):
    return [format(int(v), '08x') for v in np.asarray(a, dtype=np.float32).ravel().view(np.uint32)]


@pytest.mark.parametrize('name', ['model_be.segy', 'model_le.segy'])
def test_host_reader_matches_reference(name):
    g = _gold()[name]
    model, dims, spacing = segy.read_model_segy(os.path.join(GOLDEN, name), device=False)
    assert dims == g['dims']
    assert spacing == g['spacing']
    assert model.shape == (dims[2], dims[1], dims[0])
    assert _bits(model) == g['values_hex']


def test_header_detects_byte_order():
    be = open(os.path.join(GOLDEN, 'model_be.segy'), 'rb').read()
    le = open(os.path.join(GOLDEN, 'model_le.segy'), 'rb').read()
    assert segy.parse_header(be)[3] is True and segy.parse_header(le)[3] is False
    with pytest.raises(ValueError):
        segy.parse_header(be[:100])


def test_ibm_round_trip():
    rng = np.random.default_rng(3)
    v = (rng.standard_normal(1000) * 10.0 ** rng.integers(-20, 20, 1000)).astype(np.float32)
    back = segy.ibm_to_float(segy.float_to_ibm(v))
    assert np.all(np.abs(back - v) <= np.abs(v) * 2.0 ** -20)
    assert segy.ibm_to_float([0x80000000])[0] == 0 and not np.signbit(segy.ibm_to_float([0x80000000])[0])


def test_model_to_grid_layout():
    m = np.arange(2 * 3 * 4, dtype=np.float32).reshape(2, 3, 4)      # (nz, ny, nx)
    g = segy.model_to_grid(m, 2)
    assert g.shape == (8, 7, 6)
    assert g[2 + 3, 2 + 1, 2 + 0] == m[0, 1, 3]


@pytest.mark.gpu
@pytest.mark.parametrize('name', ['model_be.segy', 'model_le.segy'])
def test_gpu_decode_matches_reference(name):
    g = _gold()[name]
    model, dims, spacing = segy.read_model_segy(os.path.join(GOLDEN, name), device=True)
    assert dims == g['dims']
    assert _bits(model) == g['values_hex']


@pytest.mark.gpu
def test_gpu_decode_large_model(tmp_path):
    """A model larger than one block-stride pass decodes as the host does."""
    rng = np.random.default_rng(5)
    m = (1000.0 + 4000.0 * rng.random((301, 37, 29))).astype(np.float32)
    p = str(tmp_path / 'big.segy')
    segy.write_model_segy(p, m, dx=10.0, dz=5.0)
    a, dims, sp = segy.read_model_segy(p, device=True)
    b, _, _ = segy.read_model_segy(p, device=False)
    assert dims == [29, 37, 301] and sp == [10.0, 10.0, 5.0]
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    assert np.abs(a - m).max() <= np.abs(m).max() * 2.0 ** -20
