"""The reference's own model script, tests/eigenwave3d.py, run against this
package with only two edits: its Python-2 print statements become print()
calls, and the compiler it selects is 'nvcc' (given on its own command line,
``-c nvcc``).  Nothing else of the script changes.

The script is not copied into this repository: the test reads it from the
reference checkout (the OPESCI_REFERENCE environment variable, else the
directory "reference" beside this repository), applies the print edit in
memory, writes the result to a temporary directory and runs it there (the
script writes its generated program next to itself, under src/).  Without
the checkout the test is skipped.

On CPU the script's default mode runs the whole flow up to the executable:
the 100^3 eigenwave model is declared through SField/VField/StaggeredGrid,
solved, given free surfaces, its kernel AI is printed, and the generated
CUDA program is built by nvcc for sm_103a.  Executing it (-x) needs a GPU.
"""
import os
import re
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, 'opesci-fd_gb300')


def reference_dir():
    return os.environ.get('OPESCI_REFERENCE', os.path.join(os.path.dirname(ROOT), 'reference'))


_PRINT = re.compile(r'^(\s*)print (.+?)\s*$')


def py3_prints(text):
    """Python-2 print statements -> print() calls (the only source edit)."""
    out = []
    for line in text.split('\n'):
        m = _PRINT.match(line)
        out.append('%sprint(%s)' % (m.group(1), m.group(2)) if m else line)
    return '\n'.join(out)


def edited_script(tmp_path, name='eigenwave3d.py'):
    src = os.path.join(reference_dir(), 'tests', name)
    if not os.path.exists(src):
        pytest.skip('reference checkout not present')
    text = py3_prints(open(src).read())
    compile(text, name, 'exec')   # valid Python 3 after the print edit alone
    dst = tmp_path / name
    dst.write_text(text)
    (tmp_path / 'src').mkdir()
    return dst


def test_print_edit_is_the_only_change(tmp_path):
    src = os.path.join(reference_dir(), 'tests', 'eigenwave3d.py')
    if not os.path.exists(src):
        pytest.skip('reference checkout not present')
    before = open(src).read().split('\n')
    after = py3_prints('\n'.join(before)).split('\n')
    changed = [(a, b) for a, b in zip(before, after) if a != b]
    assert len(before) == len(after)
    assert changed and all(b.strip().startswith('print(') and a.strip().startswith('print ') for a, b in changed)


@pytest.mark.skipif(not (os.path.exists('/usr/local/cuda/bin/nvcc') or
                         subprocess.run(['which', 'nvcc'], capture_output=True).returncode == 0),
                    reason='needs nvcc')
def test_default_mode_builds_with_nvcc(tmp_path):
    script = edited_script(tmp_path)
    env = dict(os.environ, PYTHONPATH=PKG + os.pathsep + os.environ.get('PYTHONPATH', ''))
    # the script's own switches: VTS output, profiling with PAPI event slots
    # and Pluto tiling (a no-op for the CUDA target)
    r = subprocess.run([sys.executable, str(script), 'default', '-c', 'nvcc', '-o', '-p', '--papi-events',
                        'PAPI_TOT_CYC', '--pluto', '--tile', '4 4 32'], cwd=str(tmp_path), env=env,
                       capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    assert 'require dt < ' in r.stdout
    assert 'Compiled:' in r.stdout
    exe = tmp_path / 'src' / 'eigenwave3d'
    assert exe.exists(), r.stdout[-2000:]
    src = (tmp_path / 'src' / 'eigenwave3d.cpp').read_text()
    for s in ('ofd_write_field_vts_3d(', 'long long g_PAPI_TOT_CYC;', 'profiling->g_mflops = (float)('):
        assert s in src, s


_NORM = re.compile(r'^(\w+)_l2: ([0-9.eE+-]+)\s*$', re.M)


@pytest.mark.gpu
def test_default_mode_executes_on_gpu_and_matches_oracle(tmp_path):
    """``eigenwave3d.py default -c nvcc -x``: the generated CUDA program runs
    the 100^3, 500-step eigenwave model on the GPU through Grid.execute and
    prints the nine L2 errors from Grid.convergence; each equals the oracle's
    FP64-accumulated error of the same model within 1e-4 relative (the
    printed values carry six to seven significant digits)."""
    script = edited_script(tmp_path)
    env = dict(os.environ, PYTHONPATH=PKG + os.pathsep + ROOT + os.pathsep + os.environ.get('PYTHONPATH', ''))
    r = subprocess.run([sys.executable, str(script), 'default', '-c', 'nvcc', '-x'], cwd=str(tmp_path), env=env,
                       capture_output=True, text=True, timeout=1200)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    got = {k: float(v) for k, v in _NORM.findall(r.stdout)}
    assert len(got) == 9, r.stdout[-2000:]
    from opesci.models import eigenwave_grid
    from oracle import run as orun
    g = eigenwave_grid(grid_size=(100, 100, 100), dt=0.002, ntsteps=500, space_order=4)
    (tmp_path / 'oracle').mkdir()
    ref = orun.run(g, str(tmp_path / 'oracle'), dump=False)['l2_fp64']
    for k, v in ref.items():
        assert abs(got[k] - v) <= 1e-4 * abs(v), (k, got[k], v)


def test_read_mode_generates_a_file_model_program(tmp_path):
    """``eigenwave3d.py read``: the 195^3 model whose media come from the
    raw files RHOhomogx200, VPhomogx200 and VShomogx200 (read when the
    program runs) is declared, solved and generated as a CUDA program."""
    script = edited_script(tmp_path)
    env = dict(os.environ, PYTHONPATH=PKG + os.pathsep + os.environ.get('PYTHONPATH', ''))
    r = subprocess.run([sys.executable, str(script), 'read'], cwd=str(tmp_path), env=env,
                       capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    src = (tmp_path / 'src' / 'eigenwave3d_read.cpp').read_text()
    for name in ('RHOhomogx200', 'VPhomogx200', 'VShomogx200', 'ofd_set_media(g_handle'):
        assert name in src, name


@pytest.mark.skipif(not (os.path.exists('/usr/local/cuda/bin/nvcc') or
                         subprocess.run(['which', 'nvcc'], capture_output=True).returncode == 0),
                    reason='needs nvcc')
def test_acoustic_script_builds_with_nvcc(tmp_path):
    """The reference's acoustic model script, tests/simplewaveequation.py,
    with the same print edit: ``default -c nvcc -o -p`` declares the
    RegularGrid model, solves it and builds its CUDA program with the VTS
    output step and profiling."""
    script = edited_script(tmp_path, 'simplewaveequation.py')
    env = dict(os.environ, PYTHONPATH=PKG + os.pathsep + os.environ.get('PYTHONPATH', ''))
    r = subprocess.run([sys.executable, str(script), 'default', '-c', 'nvcc', '-o', '-p'], cwd=str(tmp_path),
                       env=env, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    assert 'Compiled:' in r.stdout and (tmp_path / 'src' / 'regular3d').exists()
    src = (tmp_path / 'src' / 'regular3d.cpp').read_text()
    for s in ('ofd_regular_create', 'ofd_write_field_vts_3d(', 'profiling->g_mflops = (float)('):
        assert s in src, s


@pytest.mark.gpu
def test_acoustic_script_executes_on_gpu_and_matches_oracle(tmp_path):
    """``simplewaveequation.py default -c nvcc -x``: the 100^3, 500-step
    model runs on the GPU through Grid.execute; its printed L2 error equals
    the oracle's within the printed digits."""
    script = edited_script(tmp_path, 'simplewaveequation.py')
    env = dict(os.environ, PYTHONPATH=PKG + os.pathsep + ROOT + os.pathsep + os.environ.get('PYTHONPATH', ''))
    r = subprocess.run([sys.executable, str(script), 'default', '-c', 'nvcc', '-x'], cwd=str(tmp_path), env=env,
                       capture_output=True, text=True, timeout=1200)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    got = {k: float(v) for k, v in _NORM.findall(r.stdout)}
    assert 'MAIN_GRID' in got, r.stdout[-2000:]
    from opesci.models import simplewave_grid
    from oracle import run as orun
    g = simplewave_grid(grid_size=(100, 100, 100), dt=0.002, tmax=1.0, space_order=4)
    (tmp_path / 'oracle').mkdir()
    want = orun.run_regular(g, str(tmp_path / 'oracle'))['l2_fp64']['MAIN_GRID']
    assert abs(got['MAIN_GRID'] - want) <= 1e-4 * abs(want), (got['MAIN_GRID'], want)
