"""ORACLE — test infrastructure only.  Nothing in the product imports this.

Compiles and runs the reference-shaped C++ program emitted by
oracle/cpp_emitter.py for a StaggeredGrid model and returns its outputs
(printed L2 norms, loop time, raw dumps of the final level).  Compiler flags
are the reference's GNU flags (opesci/compilation.py:58:
-g -O3 -fno-tree-vectorize -fopenmp), or -O3 -fopenmp with vectorisation on
when ``vectorize`` is set.
"""
import hashlib
import os
import subprocess

import numpy as np

from . import cpp_emitter, regular_emitter

# -ffp-contract=off states what g++ already does for ISO C++ on x86-64 (no
# FMA contraction), so the program rounds the same on the aarch64 GPU hosts
REF_FLAGS = ['-g', '-O3', '-fno-tree-vectorize', '-fopenmp', '-std=c++11', '-ffp-contract=off']
VEC_FLAGS = ['-O3', '-fopenmp', '-std=c++11', '-ffp-contract=off']

FIELDS = ['U', 'V', 'W', 'Txx', 'Tyy', 'Tzz', 'Txy', 'Tyz', 'Txz']


def compile_program(src, workdir, vectorize=False):
    os.makedirs(workdir, exist_ok=True)
    key = hashlib.sha1((src + str(vectorize)).encode()).hexdigest()[:16]
    cpp = os.path.join(workdir, 'oracle_%s.cpp' % key)
    exe = os.path.join(workdir, 'oracle_%s' % key)
    if not os.path.exists(exe):
        with open(cpp, 'w') as f:
            f.write(src)
        flags = VEC_FLAGS if vectorize else REF_FLAGS
        cmd = ['g++'] + flags + ['-o', exe + '.tmp', cpp, '-lm']
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError('oracle compile failed: %s\n%s' % (' '.join(cmd), r.stderr[-4000:]))
        os.replace(exe + '.tmp', exe)
    return exe


def run(grid, workdir, legacy=False, source=None, threads=None, vectorize=False, dump=True, receivers=None):
    """Emit, compile and run the oracle program for ``grid``.  Returns a dict
    with 'l2' (float-accumulated, as the reference prints), 'l2_fp64',
    'loop_seconds', 'threads' and 'fields' (final level, reference layout)."""
    workdir = os.path.abspath(workdir)
    prefix = os.path.join(workdir, "dump_") if dump else None
    src = cpp_emitter.generate(grid, legacy=legacy, dump_prefix=prefix, source=source, receivers=receivers)
    exe = compile_program(src, workdir, vectorize=vectorize)
    env = dict(os.environ)
    nthreads = threads or os.cpu_count() or 1
    env['OMP_NUM_THREADS'] = str(nthreads)
    env['OMP_PROC_BIND'] = 'close'
    r = subprocess.run([exe], capture_output=True, text=True, env=env, cwd=workdir)
    if r.returncode != 0:
        raise RuntimeError('oracle run failed (%d): %s' % (r.returncode, r.stderr[-2000:]))
    out = {'l2': {}, 'l2_fp64': {}, 'loop_seconds': None, 'threads': nthreads, 'stdout': r.stdout}
    for line in r.stdout.splitlines():
        p = line.split()
        if p and p[0] == 'loop_seconds':
            out['loop_seconds'] = float(p[1])
        elif p and p[0].endswith('_l2') and len(p) >= 3:
            out['l2'][p[0][:-3]] = float(p[1])
            out['l2_fp64'][p[0][:-3]] = float(p[2])
    if dump:
        dims = tuple(d.value for d in grid.dim)
        real = np.float64 if grid.double else np.float32
        out['fields'] = {f: np.fromfile(prefix + f + '.raw', dtype=real).reshape(dims) for f in FIELDS}
        if receivers:
            out['traces'] = np.fromfile(prefix + 'traces.raw', dtype=np.float32).reshape(
                grid.ntsteps.value, 4, len(receivers))
    return out


def run_regular(grid, workdir, threads=None, vectorize=False, dump=True):
    """Emit, compile and run the oracle program of a RegularGrid (acoustic
    scheme).  Returns 'l2', 'l2_fp64', 'loop_seconds', 'threads' and
    'levels' ({field: array[3][dim1][dim2][dim3]}, all three time levels)."""
    workdir = os.path.abspath(workdir)
    prefix = os.path.join(workdir, "rdump_") if dump else None
    src = regular_emitter.generate(grid, dump_prefix=prefix)
    exe = compile_program(src, workdir, vectorize=vectorize)
    env = dict(os.environ)
    nthreads = threads or os.cpu_count() or 1
    env['OMP_NUM_THREADS'] = str(nthreads)
    env['OMP_PROC_BIND'] = 'close'
    r = subprocess.run([exe], capture_output=True, text=True, env=env, cwd=workdir)
    if r.returncode != 0:
        raise RuntimeError('oracle run failed (%d): %s' % (r.returncode, r.stderr[-2000:]))
    out = {'l2': {}, 'l2_fp64': {}, 'loop_seconds': None, 'threads': nthreads, 'stdout': r.stdout}
    for line in r.stdout.splitlines():
        p = line.split()
        if p and p[0] == 'loop_seconds':
            out['loop_seconds'] = float(p[1])
        elif p and p[0].endswith('_l2') and len(p) >= 3:
            out['l2'][p[0][:-3]] = float(p[1])
            out['l2_fp64'][p[0][:-3]] = float(p[2])
    if dump:
        from opesci.codeprinter import ccode
        dims = (len(grid.time),) + tuple(d.value for d in grid.dim)
        real = np.float64 if grid.double else np.float32
        out['levels'] = {ccode(f.label): np.fromfile(prefix + ccode(f.label) + '.raw', dtype=real).reshape(dims)
                         for f in grid.fields}
    return out
