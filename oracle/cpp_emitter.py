"""ORACLE — test infrastructure only.  Nothing in the product imports this.

Emits the reference-shaped CPU C++/OpenMP program for a StaggeredGrid model:
the same block order, loop nests, ghost-cell sequence and t0/t1 rotation as the
reference generator, so that its output is "the reference's generated C++ on
the same inputs".  Restated from:

  opesci/templates/regular3d_tmpl.py:7-134   program blocks, extern "C" ABI, main
  opesci/templates/staggered3d_tmpl.py:9-58  parallel region and time loop
  opesci/regulargrid.py:390-496,566-619      constants, fields, loop nests
  opesci/staggeredgrid.py:522-659,728-945    media, init, sweeps, ghosts, L2

Deliberate, documented additions (harness only, outside the reference's
arithmetic):
  * fields are zero-initialised (the reference's posix_memalign memory is
    uninitialised; cells no loop writes stay at their initial value);
  * heterogeneous media are defined on the full padded grid (the reference
    averages only over the interior and then reads uninitialised memory at
    the upper interior plane and in ghost formulas);
  * an optional point source, T_ii[t1][s] -= w_i[ti]/3 after each step with
    one signal per normal stress (or one for all three), as in
    tests/src/test_ref_iso_elastic.cpp:274-290;
  * optional receivers: after each step (ghosts and source applied) U, V, W
    and (Txx + Tyy + Tzz)/3 of level t1 at given array indices, as the
    reference's driver records them (test_ref_iso_elastic.cpp:227-270),
    dumped as traces[ntsteps][4][nrec];
  * omp_get_wtime() around the time loop, FP64 error/energy sums beside the
    reference's float L2, and raw dumps of the final time level.
"""
import os
import sys

from sympy import Symbol

_HERE = os.path.dirname(os.path.abspath(__file__))
_PKG = os.path.join(os.path.dirname(_HERE), 'opesci-fd_gb300')
if _PKG not in sys.path:
    sys.path.insert(0, _PKG)

from opesci.codeprinter import ccode, ccode_eq  # noqa: E402


class _Code:
    def __init__(self):
        self.lines = []

    def add(self, s):
        self.lines.extend(s.split('\n') if isinstance(s, str) else s)

    def text(self):
        return '\n'.join(self.lines)


def _for(var, lo, hi, body):
    return ['for(int %s=%s;%s<%s;++%s){' % (var, lo, var, hi, var)] + body + ['}']


def define_constants(grid):
    """regulargrid.py:390-406."""
    out = []
    for v in grid.get_all_variables():
        val = v.value
        if isinstance(val, float):
            val = repr(val)
        if v.constant:
            out.append('const %s %s = %s;' % (v.type, v.name, val))
        else:
            out.append('%s %s = %s;' % (v.type, v.name, val))
    return out


def declare_fields(grid):
    """regulargrid.py:466-496 (zero-initialised here)."""
    arr = ''.join('[%s]' % d.name for d in grid.dim)
    vsize = len(grid.time)
    for d in grid.dim:
        vsize *= d.value
    out = []
    for f in grid.fields:
        name = ccode(f.label)
        out.append('%s *_%s_vec = (%s*) calloc(%d, sizeof(%s));' % (grid.real_t, name, grid.real_t, vsize, grid.real_t))
        out.append('%s (*%s)%s = (%s (*)%s) _%s_vec;' % (grid.real_t, name, arr, grid.real_t, arr, name))
    return out


def read_data(grid):
    """Media from raw files and effective averages (staggeredgrid.py:522-598),
    defined on the whole padded grid; upper neighbours are clamped."""
    if not grid.read:
        return []
    arr = ''.join('[%s]' % d.name for d in grid.dim[1:])
    vsize = 1
    for d in grid.dim:
        vsize *= d.value
    out = []
    media = [grid.rho, grid.vp, grid.vs] + grid.beta + [grid.lam] + grid.mu
    for m in media:
        name = ccode(m.label)
        out.append('float *_%s_vec = (float*) calloc(%d, sizeof(float));' % (name, vsize))
        out.append('float (*%s)%s = (float (*)%s) _%s_vec;' % (name, arr, arr, name))
    out.append('opesci_read_simple_binary_ptr("%s", _rho_vec, %d);' % (grid.rho_file, vsize))
    out.append('opesci_read_simple_binary_ptr("%s", _vp_vec, %d);' % (grid.vp_file, vsize))
    out.append('opesci_read_simple_binary_ptr("%s", _vs_vec, %d);' % (grid.vs_file, vsize))
    n1, n2, n3 = [d.name for d in grid.dim]
    body = [
        'const int x1 = x+1 < %s ? x+1 : x; const int y1 = y+1 < %s ? y+1 : y; const int z1 = z+1 < %s ? z+1 : z;' % (n1, n2, n3),
    ]
    loop1 = ['beta[x][y][z] = 1.0/rho[x][y][z];',
             'lambda[x][y][z] = rho[x][y][z]*(pow(vp[x][y][z], 2) - 2*pow(vs[x][y][z], 2));',
             'mu[x][y][z] = rho[x][y][z]*pow(vs[x][y][z], 2);']
    loop2 = body + [
        'beta1[x][y][z] = (beta[x][y][z] + beta[x1][y][z])/2.0;',
        'beta2[x][y][z] = (beta[x][y][z] + beta[x][y1][z])/2.0;',
        'beta3[x][y][z] = (beta[x][y][z] + beta[x][y][z1])/2.0;',
        'mu12[x][y][z] = 1.0/(0.25*(1.0/mu[x][y][z] + 1.0/mu[x1][y][z] + 1.0/mu[x][y1][z] + 1.0/mu[x1][y1][z]));',
        'mu13[x][y][z] = 1.0/(0.25*(1.0/mu[x][y][z] + 1.0/mu[x1][y][z] + 1.0/mu[x][y][z1] + 1.0/mu[x1][y][z1]));',
        'mu23[x][y][z] = 1.0/(0.25*(1.0/mu[x][y][z] + 1.0/mu[x][y1][z] + 1.0/mu[x][y][z1] + 1.0/mu[x][y1][z1]));',
    ]
    for body in (loop1, loop2):
        out += _for('x', 0, n1, _for('y', 0, n2, _for('z', 0, n3, body)))
    return out


def initialise(grid):
    """Analytic initial values at t=0 (stress) and dt/2 (velocity) on each
    field's own index range (staggeredgrid.py:612-659)."""
    m = grid.margin.value
    loop = [Symbol('_' + x.name) for x in grid.index]
    out = []
    for field in grid.fields:
        if getattr(field, 'sol', None) is None:
            continue
        body = None
        for d in range(grid.dimension - 1, -1, -1):
            i = loop[d]
            if field.staggered[d + 1]:
                i1 = ccode(grid.dim[d] - m - 1)
                expr = grid.spacing[d] * (loop[d] - grid.margin.value + 0.5)
            else:
                i1 = ccode(grid.dim[d] - m)
                expr = grid.spacing[d] * (loop[d] - grid.margin.value)
            pre = ['%s %s= %s;' % (grid.real_t, grid.index[d].name, ccode(expr))]
            if d == grid.dimension - 1:
                t0 = grid.dt.value / 2 if field.staggered[0] else 0
                sol = field.sol.subs(grid.t, t0)
                body = pre + ['%s=%s;' % (ccode(field[[0] + loop]), ccode(sol))]
            else:
                body = pre + body
            body = _for(str(i), m, i1, body)
        out += ['#pragma omp for schedule(static,1)'] + body
    return out


def _sweep(grid, fields):
    """regulargrid.py:566-619 with simple_kernel."""
    grid.create_const_dict()
    m = grid.margin.value
    idx = [grid.time[len(grid.time) - 1]] + grid.index
    body = ['%s=%s;' % (ccode(f[idx]), ccode(grid.kernel_sympy(f))) for f in fields]
    d = grid.dimension - 1
    body = ['#pragma GCC ivdep'] + _for(str(grid.index[d]), m, ccode(grid.dim[d] - m), body)
    for d in range(grid.dimension - 2, -1, -1):
        body = _for(str(grid.index[d]), m, ccode(grid.dim[d] - m), body)
    return ['#pragma omp for schedule(static,1)'] + body


def stress_loop(grid):
    return _sweep(grid, grid.sfields)


def velocity_loop(grid):
    return _sweep(grid, grid.vfields)


def _bc_stmt(grid, bc, legacy_init=False):
    if grid.read:
        bc = grid.resolve_media_params(bc)
    s = ccode_eq(bc).replace('[_t + 1]', '[_t1]').replace('[_t]', '[_t0]')
    return s + ';'


def stress_bc(grid, init=False, legacy=False):
    """Stress ghosts in the reference's field/face/side order
    (staggeredgrid.py:754-813).  ``legacy`` drops the Levander normal-stress
    recompute, like the older generator that produced benchmarks/test3d.cpp."""
    grid.create_const_dict()
    out = []
    for field in grid.sfields:
        normal = field.direction[0] == field.direction[1]
        for d in range(grid.dimension):
            if (init or legacy) and normal and field.direction[0] != d + 1:
                continue
            for side in range(2):
                if field.bc[d + 1][side] == []:
                    continue
                body = None
                for d2 in range(grid.dimension - 1, -1, -1):
                    if d2 == d:
                        continue
                    if normal and field.direction[0] != d + 1:
                        i0, i1 = grid.margin.value + 1, grid.dim[d2].value - grid.margin.value - 1
                    else:
                        i0, i1 = 0, grid.dim[d2].value
                    if body is None:
                        stmts = [_bc_stmt(grid, bc) for bc in grid.transform_bc(field, d + 1, side)]
                        body = ['#pragma GCC ivdep'] + _for(str(grid.index[d2]), i0, i1, stmts)
                    else:
                        body = _for(str(grid.index[d2]), i0, i1, body)
                out += ['#pragma omp for schedule(static,1)'] + body
    return out


def velocity_bc(grid):
    """Velocity ghosts: per face normal, the field staggered along it first
    (staggeredgrid.py:815-864)."""
    grid.create_const_dict()
    out = []
    for d in range(grid.dimension):
        seq = ([f for f in grid.vfields if f.staggered[d + 1]]
               + [f for f in grid.vfields if not f.staggered[d + 1]])
        for field in seq:
            for side in range(2):
                if not field.bc[d + 1][side]:
                    continue
                body = None
                for d2 in range(grid.dimension - 1, -1, -1):
                    if d2 == d:
                        continue
                    i0, i1 = 1, grid.dim[d2].value - 1
                    if body is None:
                        stmts = [_bc_stmt(grid, bc) for bc in grid.transform_bc(field, d + 1, side)]
                        body = ['#pragma GCC ivdep'] + _for(str(grid.index[d2]), i0, i1, stmts)
                    else:
                        body = _for(str(grid.index[d2]), i0, i1, body)
                out += ['#pragma omp for schedule(static,1)'] + body
    return out


def initialise_bc(grid, legacy=False):
    """Ghosts of the initial level: [_t1] -> [0] (staggeredgrid.py:866-879)."""
    lines = stress_bc(grid, init=True, legacy=legacy) + velocity_bc(grid)
    return [l.replace('[_t1]', '[0]') for l in lines]


def time_stepping(grid):
    """regulargrid.py:408-433."""
    return ['#pragma omp single', '{', '_t0 = (_ti)%(tp);', '_t1 = (_t0 + 1)%(tp);', '}']


def converge_test(grid):
    """L2 error vs the analytic solution at the final time, with the
    reference's float accumulator (staggeredgrid.py:892-945) and an FP64 one."""
    m = grid.margin.value
    ti = grid.ntsteps.value % 2
    loop = [Symbol('_' + x.name) for x in grid.index]
    out = []
    for field in grid.fields:
        if getattr(field, 'sol', None) is None:
            continue
        name = ccode(field.label)
        l2 = name + '_l2'
        idx = [ti] + loop
        out.append('%s %s = 0.0; double %s_d = 0.0;' % (grid.real_t, l2, l2))
        body = None
        for d in range(grid.dimension - 1, -1, -1):
            if field.staggered[d + 1]:
                i1 = ccode(grid.dim[d] - m - 1)
                expr = grid.spacing[d] * (loop[d] - grid.margin.value + 0.5)
            else:
                i1 = ccode(grid.dim[d] - m)
                expr = grid.spacing[d] * (loop[d] - grid.margin.value)
            pre = ['%s %s= %s;' % (grid.real_t, grid.index[d].name, ccode(expr))]
            if d == grid.dimension - 1:
                tn = grid.dt.value * grid.ntsteps.value
                if field.staggered[0]:
                    tn += grid.dt.value / 2.0
                err = ccode((field[idx] - field.sol.subs(grid.t, tn)) ** 2.0)
                body = pre + ['{ double _e = %s; %s += _e; %s_d += _e; }' % (err, l2, l2)]
            else:
                body = pre + body
            body = _for(str(loop[d]), m, i1, body)
        out += body
        volume = 1.0
        for sp in grid.spacing:
            volume *= sp.value
        out.append('conv->%s = pow(%s*%r, 0.5);' % (l2, l2, volume))
        out.append('conv->%s_fp64 = sqrt(%s_d*%r);' % (l2, l2, volume))
    return out


def _source_signals(source):
    """(position, wavelet) with one signal for all three normal stresses, or
    (position, (x, y, z)) with one signal each, as the reference driver reads
    xsrc/ysrc/zsrc (tests/src/test_ref_iso_elastic.cpp:100-126,274-290)."""
    pos, wav = source
    wav = list(wav)
    if wav and hasattr(wav[0], '__len__'):
        if len(wav) != 3 or len({len(w) for w in wav}) != 1:
            raise ValueError('three source signals of one length expected')
        return tuple(pos), [list(w) for w in wav]
    return tuple(pos), [wav, wav, wav]


def generate(grid, legacy=False, dump_prefix=None, source=None, timer=True, receivers=None):
    """The whole program: includes, ABI structs, opesci_execute,
    opesci_convergence, opesci_free and main (regular3d_tmpl.py:7-134)."""
    c = _Code()
    c.add(['#define M_PI 3.14159265358979323846', '#include <cassert>', '#include <cstdlib>',
           '#include <cmath>', '#include <cstdio>', '#include <cstring>', '#include <omp.h>'])
    # the raw reader of src/opesciIO.cpp:319-342 (read whole float array)
    c.add(['static int opesci_read_simple_binary_ptr(const char* f, float* a, int n){',
           '  FILE* fp = fopen(f, "rb"); if(!fp){ fprintf(stderr, "cannot open %s\\n", f); exit(-1); }',
           '  size_t r = fread(a, sizeof(float), n, fp); fclose(fp);',
           '  if((int)r != n){ fprintf(stderr, "short read %s\\n", f); exit(-1); } return 0; }'])
    names = [ccode(f.label) for f in grid.fields]
    c.add('extern "C" struct OpesciGrid { %s };' % ' '.join('%s *%s;' % (grid.real_t, n) for n in names))
    c.add('extern "C" struct OpesciConvergence { %s };' % ' '.join(
        '%s %s_l2; double %s_l2_fp64;' % (grid.real_t, n, n) for n in names))
    c.add('extern "C" struct OpesciProfiling { float g_rtime; float g_ptime; float g_mflops; double loop_seconds; };')
    if source is not None:
        (sx, sy, sz), sigs = _source_signals(source)
        for q, wav in enumerate(sigs):
            c.add('static const float _src%s[%d] = {%s};' % ('xyz'[q], len(wav),
                                                           ', '.join(repr(float(w)) + 'f' for w in wav)))
    nrec = len(receivers) if receivers is not None else 0
    if nrec:
        c.add('static float _traces[%d][4][%d];' % (grid.ntsteps.value, nrec))
    c.add('extern "C" int opesci_execute(OpesciGrid *grid, OpesciProfiling *profiling){')
    c.add(define_constants(grid))
    c.add(declare_fields(grid))
    c.add(read_data(grid))
    c.add('double _tstart = 0, _tend = 0;')
    c.add('#pragma omp parallel')
    c.add('{')
    c.add(initialise(grid))
    c.add(initialise_bc(grid, legacy=legacy))
    c.add('#pragma omp barrier')
    c.add('#pragma omp master')
    c.add('_tstart = omp_get_wtime();')
    loop = time_stepping(grid) + stress_loop(grid) + stress_bc(grid, legacy=legacy) \
        + velocity_loop(grid) + velocity_bc(grid)
    if source is not None:
        loop += ['#pragma omp single', '{',
                 'if(_ti < %d){' % len(sigs[0]),
                 '%s[_t1][%d][%d][%d] -= _srcx[_ti]/3;' % (names[3], sx, sy, sz),
                 '%s[_t1][%d][%d][%d] -= _srcy[_ti]/3;' % (names[4], sx, sy, sz),
                 '%s[_t1][%d][%d][%d] -= _srcz[_ti]/3;' % (names[5], sx, sy, sz), '}', '}']
    if nrec:
        loop += ['#pragma omp single', '{']
        for r, (x, y, z) in enumerate(receivers):
            at = '[_t1][%d][%d][%d]' % (x, y, z)
            loop += ['_traces[_ti][0][%d] = %s%s;' % (r, names[0], at),
                     '_traces[_ti][1][%d] = %s%s;' % (r, names[1], at),
                     '_traces[_ti][2][%d] = %s%s;' % (r, names[2], at),
                     '_traces[_ti][3][%d] = (%s%s + %s%s + %s%s)/3;' % (r, names[3], at, names[4], at, names[5], at)]
        loop += ['}']
    c.add(['for(int _ti=0;_ti<ntsteps;_ti++){'] + loop + ['}'])
    c.add('#pragma omp barrier')
    c.add('#pragma omp master')
    c.add('_tend = omp_get_wtime();')
    c.add('}')
    c.add('profiling->loop_seconds = _tend - _tstart;')
    c.add(['grid->%s = (%s*) %s;' % (n, grid.real_t, n) for n in names])
    if dump_prefix:
        lvl = grid.ntsteps.value % 2
        n = 1
        for d in grid.dim:
            n *= d.value
        for nm in names:
            c.add('{ FILE* fp = fopen("%s%s.raw", "wb"); fwrite(&%s[%d][0][0][0], sizeof(%s), %d, fp); fclose(fp); }'
                  % (dump_prefix, nm, nm, lvl, grid.real_t, n))
    if nrec and dump_prefix:
        c.add('{ FILE* fp = fopen("%straces.raw", "wb"); fwrite(_traces, sizeof(float), %d, fp); fclose(fp); }'
              % (dump_prefix, grid.ntsteps.value * 4 * nrec))
    c.add('return 0;')
    c.add('}')
    # convergence
    c.add('extern "C" int opesci_convergence(OpesciGrid *grid, OpesciConvergence *conv){')
    c.add(define_constants(grid))
    idxs = ''.join('[%d]' % d.value for d in grid.dim)
    for n in names:
        c.add('%s (*%s)%s = (%s (*)%s) grid->%s;' % (grid.real_t, n, idxs, grid.real_t, idxs, n))
    c.add(converge_test(grid))
    c.add('return 0;')
    c.add('}')
    c.add('extern "C" int opesci_free(OpesciGrid *grid){')
    c.add(['free(grid->%s);' % n for n in names])
    c.add('return 0;')
    c.add('}')
    c.add('int main(){')
    c.add('OpesciGrid grid; OpesciConvergence conv; OpesciProfiling profiling;')
    c.add('memset(&conv, 0, sizeof(conv));')
    c.add('opesci_execute(&grid, &profiling);')
    c.add('printf("loop_seconds\\t%.6f\\n", profiling.loop_seconds);')
    c.add('opesci_convergence(&grid, &conv);')
    for f in grid.fields:
        if getattr(f, 'sol', None) is None:
            continue
        n = ccode(f.label)
        c.add('printf("%s_l2\\t%%.10f\\t%%.12e\\n", conv.%s_l2, conv.%s_l2_fp64);' % (n, n, n))
    c.add('opesci_free(&grid);')
    c.add('return 0;')
    c.add('}')
    return c.text() + '\n'
