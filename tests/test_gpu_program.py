"""The reference's generate -> compile -> execute -> convergence flow on the
CUDA target (grid.py:59-156 with compiler='nvcc'): the emitted CUDA program
exports opesci_execute / opesci_convergence / opesci_free, is built by nvcc
against libofd and driven through ctypes, and its published fields and error
norms match the oracle (the reference-shaped C++ program)."""
import numpy as np
import pytest

from opesci.models import eigenwave_grid, layered_problem
from oracle import run as orun

FIELDS = ['U', 'V', 'W', 'Txx', 'Tyy', 'Tzz', 'Txy', 'Tyz', 'Txz']


@pytest.mark.gpu
def test_eigenwave_program_execute_and_convergence(tmp_path):
    g = eigenwave_grid(grid_size=(32, 32, 32), ntsteps=60, space_order=4)
    g.execute(str(tmp_path / 'eigenwave3d.cu'), compiler='nvcc')
    l2 = g.convergence()
    lvl = g.ntsteps.value % 2
    got = {f: g.field_array(f, lvl) for f in FIELDS}
    g.free()
    ref = orun.run(g, str(tmp_path / 'oracle'))
    state = np.sqrt(sum(np.linalg.norm(ref['fields'][f].astype(np.float64)) ** 2 for f in FIELDS))
    for f in FIELDS:
        d = np.linalg.norm(got[f].astype(np.float64) - ref['fields'][f]) / state
        assert d < 1e-5, (f, d)
        assert abs(l2[f + '_l2'] - ref['l2_fp64'][f]) <= 1e-4 * ref['l2_fp64'][f] + 1e-9, f


@pytest.mark.gpu
def test_heterogeneous_program_with_source(tmp_path):
    files = {k: str(tmp_path / (k + '.raw')) for k in ('rho', 'vp', 'vs')}
    g, media, src, wav = layered_problem(36, space_order=8, ntsteps=50, seed=4, media_files=files)
    # separate x, y and z signals, as the reference driver reads them
    sigs = ([float(v) for v in wav], [float(-0.5 * v) for v in wav], [float(v) for v in np.roll(wav, 5)])
    g.set_source(src, sigs)
    g.execute(str(tmp_path / 'layered.cu'), compiler='nvcc')
    lvl = g.ntsteps.value % 2
    got = {f: g.field_array(f, lvl) for f in FIELDS}
    g.free()
    ref = orun.run(g, str(tmp_path / 'oracle'), source=(src, sigs))
    for f in FIELDS:
        # space order 8: Robertsson ghosts and the generated update expressions
        # reproduce the reference program bit for bit
        assert np.array_equal(got[f], ref['fields'][f]), f


def test_cpu_compilers_are_rejected():
    g = eigenwave_grid(grid_size=(12, 12, 12), ntsteps=2)
    for name in ('g++', 'gnu', 'clang', 'intel'):
        with pytest.raises(ValueError, match='CPU'):
            g.compiler = name
    src = g.cgen_template.generate()
    for sym in ('opesci_execute', 'opesci_convergence', 'opesci_free', 'ofd_step', 'ofd_set_coefficients'):
        assert sym in src


def test_program_storage_and_ghost_tables():
    """double=True emits FP64 storage and double transfers; a float SO4
    Levander model passes its printed ghost equations' literals."""
    g = eigenwave_grid(grid_size=(12, 12, 12), ntsteps=3, double=True)
    src = g.cgen_template.generate()
    for s in ('typedef double real_t;', 'cfg.storage = OFD_F64;', 'ofd_upload_field_f64', 'ofd_download_field_f64'):
        assert s in src, s
    assert 'ofd_set_ghost_coefficients' not in src
    f = eigenwave_grid(grid_size=(12, 12, 12), ntsteps=3).cgen_template.generate()
    assert 'typedef float real_t;' in f and 'OFD_F32' in f and 'ofd_set_ghost_coefficients(g_handle' in f
    g8 = eigenwave_grid(grid_size=(12, 12, 12), ntsteps=3, space_order=8).cgen_template.generate()
    assert 'ofd_set_ghost_coefficients' not in g8


def test_program_profiling_fields():
    """profiling: MFlops/s from the update expressions' operation counts
    (get_kernel_ai); PAPI event slots keep the caller's struct layout."""
    g = eigenwave_grid(grid_size=(12, 12, 12), ntsteps=3)
    assert 'g_mflops = (float)(' not in g.cgen_template.generate()
    g.profiling = True
    g.set_papi_events(['PAPI_L1_DCM', 'PAPI_TOT_INS'])
    src = g.cgen_template.generate()
    v, s = g.get_velocity_kernel_ai(), g.get_stress_kernel_ai()
    assert 'g_mflops = (float)(%d.0 * pts' % (v[2] + v[3] + s[2] + s[3]) in src
    assert 'float g_mflops; long long g_PAPI_L1_DCM; long long g_PAPI_TOT_INS; };' in src
    assert 'profiling->g_PAPI_TOT_INS = 0;' in src


def test_switches_off_use_the_default_form():
    """expand=False or eval_const=False: the program runs the same update in
    the default printed form (the prebuilt kernels' form), with the printed
    ghost table of that form; the grid keeps its switches."""
    from opesci.templates import cuda_gen
    base = cuda_gen.sweep_tables(eigenwave_grid(grid_size=(12, 12, 12), ntsteps=3))
    for kw in (dict(expand=False), dict(eval_const=False), dict(expand=False, eval_const=False)):
        g = eigenwave_grid(grid_size=(12, 12, 12), ntsteps=3, **kw)
        tabs, own = cuda_gen.model_tables(g)
        assert not own and all(g.__dict__[k] is False for k in kw)
        for kind in ('stress', 'velocity'):
            assert tabs[kind][0] == base[kind][0] and np.array_equal(tabs[kind][1], base[kind][1])
        src = g.cgen_template.generate()
        assert 'ofd_set_ghost_coefficients(g_handle' in src


def test_program_source_forms():
    """One signal goes through ofd_set_source, three (x, y, z) through
    ofd_set_source_xyz; three signals of unequal length are rejected."""
    g, media, src, wav = layered_problem(16, space_order=4, ntsteps=6, seed=2)
    g.set_source(src, wav)
    one = g.cgen_template.generate()
    assert 'ofd_set_source(g_handle' in one and 'ofd_set_source_xyz' not in one
    g.set_source(src, (wav, wav * 0.5, wav))
    three = g.cgen_template.generate()
    assert 'ofd_set_source_xyz(g_handle' in three and 'src_wav[3][6]' in three
    with pytest.raises(ValueError):
        g.set_source(src, (wav, wav[:3], wav))


@pytest.mark.gpu
def test_program_output_vts(tmp_path, monkeypatch):
    """output_vts: the program writes U of the new level to U_<ti>.vts after
    every step (regulargrid.py:702-719); the first dump equals the oracle
    after one step and the last equals the published final field."""
    from opesci import vts
    monkeypatch.chdir(tmp_path)
    g = eigenwave_grid(grid_size=(24, 24, 24), ntsteps=4, space_order=4)
    g.output_vts = True
    g.profiling = True
    g.set_papi_events(['PAPI_TOT_CYC'])
    g.execute(str(tmp_path / 'eigen_vts.cu'), compiler='nvcc')
    # profiling: the time loop's CUDA-event time and MFlops/s, PAPI slot zero
    assert g._arg_profiling.rtime > 0 and g._arg_profiling.mflops > 0
    assert g._arg_profiling.PAPI_TOT_CYC == 0
    last = g.field_array('U', g.ntsteps.value % 2)
    g.free()
    dumps = [vts.read_vts(str(tmp_path / ('U_%d.vts' % t))) for t in range(4)]
    assert all(d['extent'] == tuple(last.shape) for d in dumps)
    assert np.array_equal(dumps[-1]['arrays']['field'], last.reshape(-1))
    one = eigenwave_grid(grid_size=(24, 24, 24), ntsteps=1, space_order=4)
    ref = orun.run(one, str(tmp_path / 'oracle'))
    first, want = dumps[0]['arrays']['field'].astype(np.float64), ref['fields']['U'].reshape(-1).astype(np.float64)
    assert np.linalg.norm(first - want) <= 1e-5 * np.linalg.norm(want)


@pytest.mark.gpu
def test_double_program_matches_fp64_oracle(tmp_path):
    """The double switch (regulargrid.py:27-28): FP64 storage and
    arithmetic, double fields published through OpesciGrid and double norms
    through OpesciConvergence, against the oracle built with double."""
    g = eigenwave_grid(grid_size=(24, 24, 24), ntsteps=40, space_order=4, double=True)
    g.execute(str(tmp_path / 'eigen64.cu'), compiler='nvcc')
    l2 = g.convergence()
    lvl = g.ntsteps.value % 2
    got = {f: g.field_array(f, lvl) for f in FIELDS}
    g.free()
    ref = orun.run(g, str(tmp_path / 'oracle'))
    state = np.sqrt(sum(np.linalg.norm(ref['fields'][f]) ** 2 for f in FIELDS))
    for f in FIELDS:
        assert got[f].dtype == np.float64 and ref['fields'][f].dtype == np.float64
        # FP64 storage evaluates the restated ghost formulas with exact
        # constants where the printed ones carry float (F) literals: the
        # fields differ by about 3e-9 of the state norm (measured)
        assert np.linalg.norm(got[f] - ref['fields'][f]) <= 1e-7 * state, f
        assert abs(l2[f + '_l2'] - ref['l2_fp64'][f]) <= 1e-5 * ref['l2_fp64'][f], f
