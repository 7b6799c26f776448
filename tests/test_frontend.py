"""Symbolic frontend against the reference's known answers (CPU only).

Known answers come from the reference notebooks' stored outputs
(tests/golden/notebook_outputs.json, extracted by make_golden.py):
eigenwave3d.ipynb cells 3, 11, 12, 14 and eigenwave3d-read.ipynb cells 14, 15,
24, eigenwave3d-higher_order.ipynb cell 18.
"""
import json
import os

import pytest
from sympy import Rational, Symbol, symbols, simplify, IndexedBase, Indexed, sympify

from opesci.util import staggered_weights, Taylor_half, Deriv_half
from opesci.models import elastic_grid, eigenwave_grid, stable_dt, cfl_dt

GOLDEN = os.path.join(os.path.dirname(__file__), 'golden')


@pytest.fixture(scope='module')
def grid100():
    return elastic_grid((1.0, 1.0, 1.0), (100, 100, 100), 0.002, 1.0, space_order=4)


@pytest.fixture(scope='module')
def notebooks():
    return json.load(open(os.path.join(GOLDEN, 'notebook_outputs.json')))


def test_staggered_weights_so4_so8():
    # eigenwave3d.ipynb cell 11: 9/8 and 1/24 (4th order)
    assert staggered_weights(4) == [Rational(9, 8), Rational(-1, 24)]
    assert staggered_weights(2) == [1]
    w8 = staggered_weights(8)
    assert w8 == [Rational(1225, 1024), Rational(-245, 3072), Rational(49, 5120), Rational(-5, 7168)]


def test_staggered_weights_16th_order(notebooks):
    # eigenwave3d-higher_order.ipynb cell 18: coefficients of the 16th-order
    # kernel, e.g. 41409225/33554432 and 143/167772160
    out = notebooks['eigenwave3d-higher_order.ipynb']['18']['output']
    w = staggered_weights(16)
    assert w[0] == Rational(41409225, 33554432)
    assert w[7] == Rational(-143, 167772160)
    for num in ('41409225', '3578575', '3864861', '1254825', '325325', '61425', '7425', '143'):
        assert num in out


def test_deriv_half_matches_notebook(notebooks):
    # cell 11: Txx.d[1][1].fd[4] = Txx[x-3/2]/(24dx1) - 9Txx[x-1/2]/(8dx1) + ...
    t, x, y, z, dx1 = symbols('t x y z dx1')
    T = IndexedBase('Txx')
    d = Deriv_half(T, [t, x, y, z], 1, dx1, 2)[1]
    h = Rational(1, 2)
    expect = (T[t, x - 3 * h, y, z] / (24 * dx1) - 9 * T[t, x - h, y, z] / (8 * dx1)
              + 9 * T[t, x + h, y, z] / (8 * dx1) - T[t, x + 3 * h, y, z] / (24 * dx1))
    assert simplify(d - expect) == 0
    assert '24*dx1' in notebooks['eigenwave3d.ipynb']['11']['output'].replace('⋅', '*')


def test_time_step_limit(grid100, notebooks):
    # eigenwave3d.ipynb cell 3: 0.00495
    assert abs(grid100.get_time_step_limit() - 0.00495) < 1e-12
    assert notebooks['eigenwave3d.ipynb']['3']['output'].strip() == '0.00495'
    # the same 6/7 h/(sqrt(3) Vp) rule (opesciHandy.cpp:69-89) for SO4
    assert abs(stable_dt(0.01, 1.0, 4) - 0.01 * 6 / 7 / 3 ** 0.5) < 1e-15
    assert abs(cfl_dt(0.01, 1.0, 4) - 0.5 * stable_dt(0.01, 1.0, 4)) < 1e-18


def _idx(name, *ix):
    return Indexed(IndexedBase(name), *ix)


def plain(expr):
    """Replace field/media bases by plain IndexedBase objects of the same name."""
    reps = {}
    for a in expr.atoms(Indexed):
        reps[a] = Indexed(IndexedBase(a.base.label.name), *a.indices)
    return expr.xreplace(reps)


def test_txx_kernel_aligned(grid100):
    # eigenwave3d.ipynb cell 12 (time index named _t here)
    t, x, y, z = symbols('_t x y z')
    dt, dx1, dx2, dx3, lam, mu = symbols('dt dx1 dx2 dx3 lambda mu')
    U = lambda *i: _idx('U', *i)  # noqa: E731
    V = lambda *i: _idx('V', *i)  # noqa: E731
    W = lambda *i: _idx('W', *i)  # noqa: E731
    expect = (dt * dx1 * dx2 * lam * (27 * W(t, x, y, z) + W(t, x, y, z - 2) - 27 * W(t, x, y, z - 1) - W(t, x, y, z + 1))
              + dt * dx1 * dx3 * lam * (27 * V(t, x, y, z) + V(t, x, y - 2, z) - 27 * V(t, x, y - 1, z) - V(t, x, y + 1, z))
              + dt * dx2 * dx3 * (27 * lam * U(t, x, y, z) + lam * U(t, x - 2, y, z) - 27 * lam * U(t, x - 1, y, z)
                                  - lam * U(t, x + 1, y, z) + 54 * mu * U(t, x, y, z) + 2 * mu * U(t, x - 2, y, z)
                                  - 54 * mu * U(t, x - 1, y, z) - 2 * mu * U(t, x + 1, y, z))
              + 24 * dx1 * dx2 * dx3 * _idx('Txx', t, x, y, z)) / (24 * dx1 * dx2 * dx3)
    got = grid100.sfields[0].kernel_aligned
    assert simplify(plain(got) - expect) == 0


def test_levander_velocity_ghost(grid100):
    # eigenwave3d.ipynb cell 14: U.bc[1][0][0]
    t, y, z = symbols('_t y z')
    dx1, dx2, dx3, lam, mu = symbols('dx1 dx2 dx3 lambda mu')
    eq = grid100.vfields[0].bc[1][0][0]
    assert plain(eq.lhs) == _idx('U', t + 1, 1, y, z)
    expect = (dx1 * dx2 * lam * _idx('W', t + 1, 2, y, z) - dx1 * dx2 * lam * _idx('W', t + 1, 2, y, z - 1)
              + dx1 * dx3 * lam * _idx('V', t + 1, 2, y, z) - dx1 * dx3 * lam * _idx('V', t + 1, 2, y - 1, z)
              + dx2 * dx3 * lam * _idx('U', t + 1, 2, y, z) + 2 * dx2 * dx3 * mu * _idx('U', t + 1, 2, y, z)
              ) / (dx2 * dx3 * (lam + 2 * mu))
    assert simplify(plain(eq.rhs) - expect) == 0


def test_kernel_ai_counts(grid100, notebooks):
    # Operation counts of the expanded, constant-folded SO4 kernels.  They
    # equal the tuples stored in eigenwave3d-read.ipynb cells 14-15.  The
    # older eigenwave3d.ipynb (cells 18-19) shows exactly twice these ADD/MUL
    # counts: its SymPy version did not combine like terms after folding.
    assert grid100.get_velocity_kernel_ai() == (1.5, 1.5, 36, 36, 9, 3)
    assert grid100.get_stress_kernel_ai() == (2.0, 2.0, 60, 60, 9, 6)
    rd = notebooks['eigenwave3d-read.ipynb']
    assert rd['14']['output'].strip() == '(1.5, 1.5, 36, 36, 9, 3)'
    assert rd['15']['output'].strip() == '(2.0, 2.0, 60, 60, 9, 6)'
    ew = notebooks['eigenwave3d.ipynb']
    assert ew['18']['output'].strip() == '(3.0, 3.0, 72, 72, 9, 3)'


def test_read_mode_mu12_ghost(notebooks):
    # eigenwave3d-read.ipynb cell 24: U ghost on the lower y face resolved to mu12
    from opesci.codeprinter import ccode
    g = elastic_grid((1.0, 1.0, 1.0), (20, 20, 20), 0.002, 0.01, space_order=4, read=True,
                     rho_file='r', vp_file='p', vs_file='s', analytic=False)
    got = ccode(g.resolve_media_params(g.vfields[0].bc[2][0][0]))
    ref = notebooks['eigenwave3d-read.ipynb']['24']['output'].strip().strip("'")
    parse = lambda s: sympify(s.split(' = ')[1].replace('][', ',').replace('[', '(').replace(']', ')')  # noqa: E731
                              .replace('_t', 't').replace('lambda', 'lam'))
    assert simplify(parse(got) - parse(ref)) == 0
    assert got.split(' = ')[0].replace('_t', 't') == ref.split(' = ')[0]


def test_python2_division_semantics():
    # Taylor(): range(-n/2, n/2+1) with Python-2 floor division
    from opesci.util import Taylor
    assert Taylor(Symbol('h'), 3).shape == (4, 4)     # rows -2..1
    assert Taylor_half(Symbol('h'), 2).shape == (4, 4)


def test_margins_and_dims():
    g = eigenwave_grid(grid_size=(16, 16, 16), ntsteps=3, space_order=8)
    assert g.margin.value == 4
    assert [d.value for d in g.dim] == [25, 25, 25]
    assert abs(g.spacing[0].value - 1.0 / 16) < 1e-15
    assert g.fields[0].label.name == 'U' and g.fields[3].label.name == 'Txx'
    assert g.free_surface[(1, 0)] == 'robertsson'
    g4 = eigenwave_grid(grid_size=(16, 16, 16), ntsteps=3, space_order=4)
    assert g4.free_surface[(3, 1)] == 'levander'


def test_switch_validation(grid100):
    with pytest.raises(KeyError):
        grid100.set_switches(nonsense=True)
    with pytest.raises(ValueError):
        grid100.set_switches(omp=1)
    with pytest.raises(ValueError):
        grid100.set_order([2, 3, 3, 3])
