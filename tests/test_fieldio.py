"""Raw field files (the reference's dump/read format) and checkpoints that
resume a device-resident run bit for bit."""
import numpy as np
import pytest

from opesci import batch, fieldio, runtime


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
