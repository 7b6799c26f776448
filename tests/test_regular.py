"""The regular-grid (acoustic) scheme of RegularGrid: the reference's model
tests/simplewaveequation.py:9-81, its three-level time loop
(regulargrid.py:408-433,566-619) and its initialisation
(regulargrid.py:498-564).

CPU: the frontend's term table (the form the device sweep evaluates) is
checked against the oracle, the reference-shaped C++ program compiled by
g++: one step evaluated from the table in float32, term by term in table
order, equals the oracle's step bit for bit.  The generated CUDA program
cross-compiles.  GPU: the device runtime and the generated program reproduce
the oracle's three time levels bit for bit.

Parity of the acoustic program is not pinned by a reference output: the
reference holds no generated acoustic program or printed result.  The
oracle restates the reference generator's program blocks for it."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from opesci.models import simplewave_grid
from opesci.templates.regular_tmpl import regular_terms, split_terms
from oracle import run as orun


def _step_from_table(terms, cur, prev, m, dtype):
    """u[t+1] on the interior from the table: acc = c0*v0; acc = acc + ck*vk,
    each product and sum rounded to ``dtype``."""
    n1, n2, n3 = cur.shape
    sl = lambda a, o: a[m + o[0]:n1 - m + o[0], m + o[1]:n2 - m + o[1], m + o[2]:n3 - m + o[2]]  # noqa: E731
    acc = None
    for lvl, off, coef in terms:
        p = (dtype(coef) * sl(cur if lvl else prev, off)).astype(dtype)
        acc = p if acc is None else (acc + p).astype(dtype)
    return acc


def test_split_terms_respects_brackets():
    t = split_terms('-A[_t0][x][y + 1][z] + 2.0e-1F*A[_t1][x - 2][y][z] - 3*A[_t1][x][y][z + 1]')
    assert t == [(-1, 'A[_t0][x][y + 1][z]'), (1, '2.0e-1F*A[_t1][x - 2][y][z]'), (-1, '3*A[_t1][x][y][z + 1]')]


@pytest.mark.parametrize('so', [2, 4, 8])
def test_term_table_matches_reference_program(tmp_path, so):
    g = simplewave_grid(grid_size=(18, 14, 22), space_order=so, ntsteps=6)
    terms = regular_terms(g, g.fields[0])
    # the model's equation: y twice, no z second derivative
    assert all(off[2] == 0 for _, off, _ in terms)
    assert sum(1 for lvl, _, _ in terms if lvl == 0) == 1
    r6 = orun.run_regular(g, str(tmp_path / 'a'), threads=2)['levels']['MAIN_GRID']
    g.ntsteps.value = 7
    r7 = orun.run_regular(g, str(tmp_path / 'b'), threads=2)['levels']['MAIN_GRID']
    m = g.margin.value
    # step _ti = 6: _t0 = 0, _t1 = 1, writes level 2
    got = _step_from_table(terms, r6[1], r6[0], m, np.float32)
    want = r7[2][m:-m, m:-m, m:-m]
    assert np.array_equal(got, want)
    assert np.abs(want).max() > 0


def test_coefficient_values_follow_c_literals():
    """Coefficients take the value the C compiler gives the printed literal:
    float literals rounded once to float32, integers exactly, p.0F/q.0F as a
    float32 division."""
    from fractions import Fraction
    from opesci.templates.regular_tmpl import _coef_value
    for lit in ('2.13333333333333e-1', '1.33333333333333e-2', '8.0e-1', '1.06666666666667e-1'):
        f = _coef_value(lit + 'F')
        q = Fraction(lit)
        up = np.nextafter(f, np.float32(np.inf))
        down = np.nextafter(f, np.float32(-np.inf))
        # nearest float32 to the decimal value
        assert abs(Fraction(float(f)) - q) <= min(abs(Fraction(float(up)) - q), abs(Fraction(float(down)) - q))
    assert _coef_value('2') == np.float32(2)
    assert _coef_value('1.0F/12.0F') == np.float32(1) / np.float32(12)
    with pytest.raises(ValueError):
        _coef_value('dt')


def test_fp64_table_keeps_float_literals():
    """With double=True the printed literals still carry the F suffix, so the
    FP64 program multiplies by float32 values; the table is the FP32 one."""
    a = regular_terms(*(lambda g: (g, g.fields[0]))(simplewave_grid(grid_size=(12, 12, 12), ntsteps=2)))
    b = regular_terms(*(lambda g: (g, g.fields[0]))(simplewave_grid(grid_size=(12, 12, 12), ntsteps=2,
                                                                   double=True)))
    assert a == b
    assert all(float(np.float32(c)) == c for _, _, c in a)


def test_term_table_rejects_unexpanded_kernels():
    g = simplewave_grid(grid_size=(10, 10, 10), space_order=4, ntsteps=2)
    g.expand = False
    with pytest.raises(ValueError, match='expand'):
        regular_terms(g, g.fields[0])


def test_switches_off_use_the_default_form():
    """With expand or eval_const off the device runs the same update in the
    default printed form; the grid's switches are left as they were."""
    from opesci.templates.regular_tmpl import model_terms
    ref = regular_terms(simplewave_grid(grid_size=(10, 10, 10), space_order=4, ntsteps=2),
                        simplewave_grid(grid_size=(10, 10, 10), space_order=4, ntsteps=2).fields[0])
    for sw in ('expand', 'eval_const'):
        g = simplewave_grid(grid_size=(10, 10, 10), space_order=4, ntsteps=2)
        setattr(g, sw, False)
        assert model_terms(g, g.fields[0]) == ref
        assert getattr(g, sw) is False
        assert 'ofd_regular_create' in g.cgen_template.generate()


def test_oracle_second_initialisation(tmp_path):
    """The reference's second initialisation with v = 1 on a zero level 0
    gives level 1 = v*dt on the interior, zero on the margins."""
    g = simplewave_grid(grid_size=(12, 12, 12), space_order=4, ntsteps=0)
    lv = orun.run_regular(g, str(tmp_path), threads=2)['levels']['MAIN_GRID']
    m = g.margin.value
    assert not lv[0].any() and not lv[2].any()
    assert np.all(lv[1][m:-m, m:-m, m:-m] == np.float32(np.float32(1.0) * np.float32(0.002)))
    assert not lv[1][:m].any() and not lv[1][-m:].any()


@pytest.mark.skipif(shutil.which('nvcc') is None and not os.path.exists('/usr/local/cuda/bin/nvcc'),
                    reason='nvcc not available')
def test_generated_program_compiles(tmp_path):
    from opesci import build
    lib = build.build()
    for double in (False, True):
        g = simplewave_grid(grid_size=(16, 16, 16), space_order=4, ntsteps=3, double=double)
        # with the output_vts and profiling switches: the per-step VTS dump
        # and the MFlops/s figure are compiled in as well
        g.output_vts = double
        g.profiling = double
        src = g.cgen_template.generate()
        assert ('ofd_write_field_vts_3d(' in src) == double and ('g_mflops = (float)(' in src) == double
        for sym in ('opesci_execute', 'opesci_convergence', 'opesci_free', 'ofd_regular_create', 'ofd_regular_step'):
            assert sym in src
        cu = tmp_path / ('simplewave_%d.cu' % double)
        cu.write_text(src)
        nvcc = shutil.which('nvcc') or '/usr/local/cuda/bin/nvcc'
        cmd = [nvcc, '-gencode', 'arch=compute_103a,code=sm_103a', '-O3', '-std=c++17', '-fmad=false',
               '-I', build.INCLUDE, '-Xcompiler', '-fPIC', '-shared', '-o', str(cu) + '.so', str(cu),
               '-L', os.path.dirname(lib), '-lofd']
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-3000:]


# ----------------------------------------------------------------- GPU

def _levels_sim(g, ref0, variant=0):
    """RegularSimulation holding the oracle's initial levels."""
    from opesci import runtime
    sim = runtime.RegularSimulation(runtime.regular_config_from_grid(g, variant=variant))
    for lvl in range(3):
        sim.upload(lvl, ref0[lvl])
    return sim


@pytest.mark.gpu
@pytest.mark.parametrize('variant', [0, 1])
@pytest.mark.parametrize('so,double,shape', [(2, False, (37, 29, 45)), (4, False, (37, 29, 45)),
                                             (8, False, (33, 41, 30)), (4, True, (25, 31, 27)),
                                             (16, False, (40, 24, 36))])
def test_device_sweep_matches_oracle(tmp_path, so, double, shape, variant):
    g = simplewave_grid(grid_size=shape, space_order=so, ntsteps=0, double=double)
    ref0 = orun.run_regular(g, str(tmp_path / 'r0'), threads=4)['levels']['MAIN_GRID']
    steps = 11
    g.ntsteps.value = steps
    ref = orun.run_regular(g, str(tmp_path / 'rn'), threads=4)['levels']['MAIN_GRID']
    sim = _levels_sim(g, ref0, variant)
    sim.step(steps)
    sim.sync()
    assert sim.steps == steps
    for lvl in range(3):
        got = sim.download(lvl)
        assert np.array_equal(got, ref[lvl]), (lvl, float(np.abs(got - ref[lvl]).max()))
    sim.close()


@pytest.mark.gpu
def test_reference_default_case_program(tmp_path):
    """tests/simplewaveequation.py default mode: 100^3 unit cube, order
    [2, 4, 4, 4], dt = 0.002, tmax = 1.0 (500 steps), through
    generate -> nvcc -> execute -> convergence."""
    g = simplewave_grid(grid_size=(100, 100, 100), dt=0.002, tmax=1.0, space_order=4)
    assert g.ntsteps.value == 500
    g.execute(str(tmp_path / 'simplewave3d.cu'), compiler='nvcc')
    l2 = g.convergence()
    got = g.field_array('MAIN_GRID')
    g.free()
    ref = orun.run_regular(g, str(tmp_path / 'oracle'))
    for lvl in range(3):
        assert np.array_equal(got[lvl], ref['levels']['MAIN_GRID'][lvl]), lvl
    want = ref['l2_fp64']['MAIN_GRID']
    assert abs(l2['MAIN_GRID_l2'] - want) <= 1e-5 * want


@pytest.mark.gpu
def test_eval_const_off_matches_oracle(tmp_path):
    """eval_const off: the device runs the default printed form; the oracle
    evaluates the named constants at run time (the two forms differ by
    ~5e-7 relative after 10 steps, oracle against oracle).  Each level within
    1e-5 relative L2."""
    g = simplewave_grid(grid_size=(30, 26, 28), space_order=4, ntsteps=0)
    g.eval_const = False
    ref0 = orun.run_regular(g, str(tmp_path / 'r0'), threads=4)['levels']['MAIN_GRID']
    g.ntsteps.value = 10
    ref = orun.run_regular(g, str(tmp_path / 'rn'), threads=4)['levels']['MAIN_GRID']
    sim = _levels_sim(g, ref0)
    sim.step(10)
    sim.sync()
    for lvl in range(3):
        a, b = sim.download(lvl).astype(np.float64), ref[lvl].astype(np.float64)
        assert np.linalg.norm(a - b) <= 1e-5 * np.linalg.norm(b), lvl
    sim.close()
    assert g.eval_const is False


@pytest.mark.gpu
def test_program_output_vts(tmp_path, monkeypatch):
    """output_vts: the new level after every step in MAIN_GRID_<ti>.vts
    (regulargrid.py:702-719); the last dump is the published level
    (ntsteps + 1) % 3."""
    from opesci import vts
    monkeypatch.chdir(tmp_path)
    g = simplewave_grid(grid_size=(20, 20, 20), dt=0.002, space_order=4, ntsteps=4)
    g.output_vts = True
    g.execute(str(tmp_path / 'simplewave_vts.cu'), compiler='nvcc')
    got = g.field_array('MAIN_GRID')
    g.free()
    ref = orun.run_regular(g, str(tmp_path / 'oracle'))['levels']['MAIN_GRID']
    last = vts.read_vts(str(tmp_path / 'MAIN_GRID_3.vts'))
    assert np.array_equal(last['arrays']['field'], got[5 % 3].reshape(-1))
    assert np.array_equal(last['arrays']['field'], ref[5 % 3].reshape(-1))
    assert all((tmp_path / ('MAIN_GRID_%d.vts' % t)).exists() for t in range(4))


def test_device_config_validation_without_gpu():
    """ofd_regular_create checks its configuration before touching the GPU."""
    from opesci import build, runtime
    build.build()
    for cfg, msg in ((runtime.regular_config((20, 20, 20), 2, [(1, (3, 0, 0), 1.0)]), 'margin'),
                     (runtime.regular_config((20, 20, 20), 9, [(1, (0, 0, 0), 1.0)]), 'margin'),
                     (runtime.regular_config((4, 20, 20), 2, [(1, (0, 0, 0), 1.0)]), 'interior'),
                     (runtime.regular_config((20, 20, 20), 2, [(1, (0, 0, 0), 1.0)], variant=2), 'variant')):
        with pytest.raises(runtime.OFDError, match=msg):
            runtime.RegularSimulation(cfg)
    with pytest.raises(ValueError):
        runtime.regular_config((20, 20, 20), 2, [(1, (0, 0, 0), 1.0)], storage='f16')
