"""Finite-difference helpers: Taylor matrices, staggered/regular derivative
stencils, expression walkers and operation counters.

Restates the helpers of opesci/util.py (reference). Python-2 integer division
in the reference (``-n/2``) is written as floor division here.
"""
from sympy import Expr, Symbol, Indexed, Rational, IndexedBase, factorial, Matrix
from sympy.core.relational import Relational

__all__ = ['hf', 'get_all_objects', 'variable_to_symbol', 'get_ops_expr',
           'IndexedBases', 'tc', 'Taylor', 'Taylor_half', 'Taylor_generic',
           'Deriv', 'Deriv_generic', 'Deriv_half', 'is_half', 'shift_grid',
           'shift_index', 'staggered_weights']

hf = Rational(1, 2)


def get_all_objects(expr, typ):
    """All sub-expressions of ``expr`` of type ``typ`` (util.py:7-20)."""
    if isinstance(expr, typ):
        return [expr]
    # Equalities are traversed too: the reference walks Eq objects when it
    # substitutes stencils into the PDEs (staggeredgrid.py:155).
    if not isinstance(expr, (Expr, Relational)):
        return []
    result = []
    for arg in expr.args:
        result += get_all_objects(arg, typ)
    return result


def variable_to_symbol(variables):
    """Plain Symbols with the names of ``variables`` (util.py:23-27)."""
    return [Symbol(v.name) for v in variables]


def get_ops_expr(expr, arrays):
    """Count (ADD, MUL) in ``expr`` and collect array names (util.py:30-64).

    An n-ary Add/Mul counts n-1 operations; subtraction and division are
    folded into Add/Mul by SymPy and counted the same way."""
    if isinstance(expr, Indexed):
        base = str(expr.base.label)
        if base not in arrays:
            arrays += [base]
        return (0, 0, arrays)
    mul = 0
    add = 0
    if expr.is_Mul or expr.is_Add:
        args = expr.args
        if expr.is_Mul:
            mul += len(args) - 1
        else:
            add += len(args) - 1
        arrays2 = arrays
        for expr2 in args:
            add2, mul2, arrays2 = get_ops_expr(expr2, arrays2)
            add += add2
            mul += mul2
        return (add, mul, arrays2)
    return (0, 0, arrays)


def IndexedBases(s):
    """Several IndexedBase objects from a whitespace separated string."""
    return tuple(IndexedBase(x) for x in s.split())


def tc(dx, n):
    """Taylor coefficient dx**n / n! (util.py:78-84)."""
    return (dx ** n) / factorial(n)


def Taylor(dx, n):
    """Taylor matrix on a regular grid, rows at offsets -n/2..n/2
    (util.py:87-100; Python-2 floor division kept)."""
    rows = []
    for i in range((-n) // 2, n // 2 + 1):
        rows.append([tc(i * dx, j) for j in range(n + 1)])
    return Matrix(rows)


def Taylor_half(dx, n):
    """Taylor matrix on a staggered grid: rows at offsets (2i+1)/2 * dx for
    the 2n neighbours -(2n-1)/2 .. (2n-1)/2 (util.py:103-118)."""
    rows = []
    for i in range(-n * 2 + 1, n * 2, 2):
        rows.append([tc(i * dx / 2, j) for j in range(2 * n)])
    return Matrix(rows)


def Taylor_generic(delta, left, right, half=False):
    """Taylor matrix for neighbours -left..right, optionally shifted by 1/2
    (util.py:121-133)."""
    rows = []
    n = left + right + 1
    shift = hf if half else 0
    for i in range(-left, right + 1):
        rows.append([tc((i + shift) * delta, j) for j in range(n)])
    return Matrix(rows)


def _shifted(U, index, mask, amount):
    idx = [index[k] + mask[k] * amount for k in range(len(index))]
    return U[idx]


def Deriv(U, index, k, d, n):
    """Regular-grid FD approximations of all derivatives of order <= n
    along index k (util.py:136-173)."""
    if len(index) > 4:
        raise NotImplementedError(">4 dimensions, need to fix")
    M = Taylor(d, n)
    s = [0] * len(index)
    s[k] = 1
    RX = Matrix([_shifted(U, index, s, x) for x in range((-n) // 2, n // 2 + 1)])
    return M.inv() * RX


def Deriv_generic(U, index, dimension, delta, left, right, half=False):
    """Generic FD approximations on an arbitrary neighbour set
    (util.py:176-192)."""
    M = Taylor_generic(delta, left, right, half)
    shift = hf if half else 0
    ll = []
    for i in range(-left, right + 1):
        index2 = list(index)
        index2[dimension] = index[dimension] + i + shift
        ll.append(U[index2])
    return M.inv() * Matrix(ll)


def Deriv_half(U, index, dimension, delta, order):
    """Staggered-grid FD approximations (util.py:195-236).

    ``order`` is half the accuracy: order=2 gives the 4th-order stencil on
    the neighbours at +-1/2 and +-3/2.  Entry [1] of the result is the first
    derivative."""
    if len(index) > 4:
        raise NotImplementedError(">4 dimensions, need to fix")
    M = Taylor_half(delta, order)
    mask = [0] * len(index)
    mask[dimension] = 1
    RX = Matrix([_shifted(U, index, mask, x * hf)
                 for x in range(-order * 2 + 1, order * 2, 2)])
    return M.inv() * RX


def staggered_weights(order):
    """Weights c_1..c_R of the staggered first derivative of accuracy
    ``order`` (= 2R): f'(x) ~ sum_k c_k (f(x+(k-1/2)h) - f(x-(k-1/2)h)) / h.

    Obtained from the same Taylor-matrix inverse as Deriv_half (util.py:103-118,
    195-236); returned as exact Rationals."""
    R = order // 2
    h = Symbol('h')
    M = Taylor_half(h, R)
    row = M.inv()[1, :]
    # columns correspond to offsets -(2R-1)/2 .. (2R-1)/2
    weights = []
    for k in range(1, R + 1):
        col = R - 1 + k           # offset +(k-1/2)
        w = (row[col] * h).simplify()
        weights.append(Rational(w))
    return weights


def is_half(expr):
    """True when the constant part of an index is integer + 1/2
    (util.py:239-247)."""
    d = {x: 0 for x in expr.free_symbols}
    return not expr.subs(d).is_Integer


def shift_grid(expr):
    """Shift half indices down to whole numbers (util.py:250-267)."""
    if expr.is_Symbol or expr.is_Number:
        return expr
    if isinstance(expr, Indexed):
        idx = [x - hf if is_half(x) else x for x in list(expr.indices)]
        return Indexed(expr.base, *idx)
    args = tuple(shift_grid(arg) for arg in expr.args)
    return expr.func(*args)


def shift_index(expr, k, s):
    """Shift the k-th index of every array in ``expr`` by s
    (util.py:270-292)."""
    if expr.is_Symbol or expr.is_Number:
        return expr
    if isinstance(expr, Indexed):
        idx = list(expr.indices)
        idx[k] += s
        return Indexed(expr.base, *idx)
    args = tuple(shift_index(arg, k, s) for arg in expr.args)
    return expr.func(*args)
