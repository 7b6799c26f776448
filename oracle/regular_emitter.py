"""ORACLE — test infrastructure only.  Nothing in the product imports this.

Emits the reference-shaped CPU C++/OpenMP program of a RegularGrid (the
acoustic scheme): the block order, loop nests, initialisation and three-level
_t0/_t1/_t2 rotation of the reference's generator.  Restated from:

  opesci/templates/regular3d_tmpl.py:7-134   program blocks, extern "C" ABI, main
  opesci/regulargrid.py:390-433              constants, time stepping
  opesci/regulargrid.py:466-496              field declaration
  opesci/regulargrid.py:498-564              first and second initialisation
  opesci/regulargrid.py:566-619              primary loop (simple_kernel)
  opesci/regulargrid.py:650-700              convergence (L2 of level ntsteps % 2)

The symbolic expressions (update kernel, initialisations, analytic solution)
come from the frontend's restated generator (RegularGrid.kernel_sympy,
initial_kernel, second_initial_kernel), printed with the same C printer.

Deliberate, documented additions (harness only, outside the reference's
arithmetic):
  * the field is zero-initialised (the reference's posix_memalign memory is
    uninitialised, and nothing writes the margins of levels 1 and 2);
  * omp_get_wtime() around the time loop, an FP64 error sum beside the
    reference's float L2, and raw dumps of all three time levels;
  * the reference's convergence block also prints each spacing through a
    "%d" format; those lines are left out.
"""
from sympy import Symbol

from .cpp_emitter import _Code, _for, define_constants, declare_fields, ccode


def initialise(grid):
    """regulargrid.py:498-564: level 0 on [0, dim) from the analytic solution
    at t = 0 with loop indices for coordinates, then level _t1 on the
    interior from the second-initialisation expression."""
    loop = [Symbol('_' + x.name) for x in grid.index]
    m = grid.margin.value
    out = []
    for field in grid.fields:
        body = ['%s = %s;' % (ccode(field[[0] + loop]), ccode(grid.initial_kernel(field)))]
        for d in range(grid.dimension - 1, -1, -1):
            body = _for(str(loop[d]), 0, ccode(grid.dim[d]), body)
        out += ['#pragma omp for schedule(static,1)'] + body
        body = ['%s = %s;' % (ccode(field[[grid.time[1]] + loop]), ccode(grid.second_initial_kernel(field)))]
        for d in range(grid.dimension - 1, -1, -1):
            body = _for(str(loop[d]), m, ccode(grid.dim[d] - m), body)
        out += ['#pragma omp for schedule(static,1)'] + body
    return out


def time_stepping(grid):
    """regulargrid.py:408-433 for any number of time levels."""
    names = [t.name for t in grid.time]
    out = ['#pragma omp single', '{', '%s = (_ti)%%(tp);' % names[0]]
    for i in range(1, len(names)):
        out.append('%s = (%s + 1)%%(tp);' % (names[i], names[i - 1]))
    return out + ['}']


def primary_loop(grid):
    """regulargrid.py:566-619 with simple_kernel."""
    grid.create_const_dict()
    m = grid.margin.value
    idx = [grid.time[len(grid.time) - 1]] + grid.index
    body = ['%s = %s;' % (ccode(f[idx]), ccode(grid.kernel_sympy(f))) for f in grid.fields]
    d = grid.dimension - 1
    body = ['#pragma GCC ivdep'] + _for(str(grid.index[d]), m, ccode(grid.dim[d] - m), body)
    for d in range(grid.dimension - 2, -1, -1):
        body = _for(str(grid.index[d]), m, ccode(grid.dim[d] - m), body)
    return ['#pragma omp for schedule(static,1)'] + body


def converge_test(grid):
    """regulargrid.py:650-700: L2 of level ntsteps % 2 against the analytic
    solution at t = dt*ntsteps, with the reference's float accumulator and an
    FP64 one."""
    m = grid.margin.value
    ti = grid.ntsteps.value % 2
    loop = [Symbol('_' + x.name) for x in grid.index]
    out = []
    for field in grid.fields:
        if getattr(field, 'sol', None) is None:
            continue
        name = ccode(field.label)
        l2 = name + '_l2'
        out.append('%s %s = 0.0; double %s_d = 0.0;' % (grid.real_t, l2, l2))
        tn = grid.dt.value * grid.ntsteps.value
        err = ccode((field[[ti] + loop] - field.sol.subs(grid.t, tn)) ** 2.0)
        body = None
        for d in range(grid.dimension - 1, -1, -1):
            pre = ['%s %s = %s;' % (grid.real_t, grid.index[d].name,
                                    ccode(grid.spacing[d] * (loop[d] - grid.margin.value)))]
            if body is None:
                body = pre + ['{ double _e = %s; %s += _e; %s_d += _e; }' % (err, l2, l2)]
            else:
                body = pre + body
            body = _for(str(loop[d]), m, ccode(grid.dim[d] - m), body)
        out += body
        volume = 1.0
        for sp in grid.spacing:
            volume *= sp.value
        out.append('conv->%s = pow(%s*%r, 0.5);' % (l2, l2, volume))
        out.append('conv->%s_fp64 = sqrt(%s_d*%r);' % (l2, l2, volume))
    return out


def generate(grid, dump_prefix=None):
    """The whole program (regular3d_tmpl.py:7-134)."""
    c = _Code()
    c.add(['#define M_PI 3.14159265358979323846', '#include <cstdlib>', '#include <cmath>',
           '#include <cstdio>', '#include <cstring>', '#include <omp.h>'])
    names = [ccode(f.label) for f in grid.fields]
    c.add('extern "C" struct OpesciGrid { %s };' % ' '.join('%s *%s;' % (grid.real_t, n) for n in names))
    c.add('extern "C" struct OpesciConvergence { %s };' % ' '.join(
        '%s %s_l2; double %s_l2_fp64;' % (grid.real_t, n, n) for n in names))
    c.add('extern "C" struct OpesciProfiling { float g_rtime; float g_ptime; float g_mflops; double loop_seconds; };')
    c.add('extern "C" int opesci_execute(OpesciGrid *grid, OpesciProfiling *profiling){')
    c.add(define_constants(grid))
    c.add(declare_fields(grid))
    c.add('double _tstart = 0, _tend = 0;')
    c.add('#pragma omp parallel')
    c.add('{')
    c.add(initialise(grid))
    c.add('#pragma omp barrier')
    c.add('#pragma omp master')
    c.add('_tstart = omp_get_wtime();')
    c.add(['for(int _ti=0;_ti<ntsteps;_ti++){'] + time_stepping(grid) + primary_loop(grid) + ['}'])
    c.add('#pragma omp barrier')
    c.add('#pragma omp master')
    c.add('_tend = omp_get_wtime();')
    c.add('}')
    c.add('profiling->loop_seconds = _tend - _tstart;')
    c.add(['grid->%s = (%s*) %s;' % (n, grid.real_t, n) for n in names])
    if dump_prefix:
        n = len(grid.time)
        for d in grid.dim:
            n *= d.value
        for nm in names:
            c.add('{ FILE* fp = fopen("%s%s.raw", "wb"); fwrite(&%s[0][0][0][0], sizeof(%s), %d, fp); fclose(fp); }'
                  % (dump_prefix, nm, nm, grid.real_t, n))
    c.add('return 0;')
    c.add('}')
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
