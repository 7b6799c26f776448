"""Staggered-grid fields: velocity (VField), stress (SField), media (Media).

Restates opesci/fields.py (reference) for SymPy 1.14 / Python 3:
single-argument ``Eq(x)`` becomes ``Eq(x, 0)`` and Python-2 integer division
becomes floor division.  Free-surface ghost equations follow fields.py:192-381
(Robertsson 1996 zero-velocity ghosts; Levander 1988 zero-traction ghosts for
4th-order schemes).
"""
from sympy import Indexed, IndexedBase, solve, Eq, Symbol
from .util import hf, Deriv_half, Deriv, get_all_objects
from .derivative import DDerivative

__all__ = ['SField', 'VField', 'Media', 'RegularField', 'Field']

# SymPy rebuilds IndexedBase objects from their args (label only) while
# substituting or solving.  The rebuilt object must be the instance that holds
# the staggering information, so bare reconstructions are routed to the last
# instance created with that label and class.
_registry = {}


class Field(IndexedBase):
    """A field on the staggered grid, indexable as F[t, x, y, z].

    Holds the dimension, the staggering flags (one per index, time first),
    the derivative table ``d[index][order]`` with its FD approximations, the
    update kernel and the free-surface ghost equations ``bc[dim][side]``
    (fields.py:8-166)."""

    def __new__(cls, name, *args, **kwargs):
        label = name.name if isinstance(name, Symbol) else str(name)
        key = (cls, label)
        if not kwargs and key in _registry:
            return _registry[key]
        obj = IndexedBase.__new__(cls, label)
        if kwargs:
            _registry[key] = obj
        return obj

    def __init__(self, *args, **kwargs):
        if len(kwargs) > 1:
            self.set(**kwargs)

    def __getnewargs_ex__(self):
        return ((self.label.name,), {})

    def set(self, dimension, staggered):
        self.dimension = dimension
        self.staggered = staggered
        self.bc = [[None] * 2 for _ in range(dimension + 1)]

    def set_analytic_solution(self, function):
        """Exact solution used for initial values and error norms."""
        self.sol = function

    def set_indices(self, indices):
        """Index symbols, e.g. [t, x, y, z]."""
        self.indices = indices

    def set_spacing(self, spacing):
        """Spacing symbols, e.g. [dt, dx1, dx2, dx3]."""
        self.spacing = spacing

    def set_order(self, order):
        """Accuracy per index, e.g. [2, 4, 4, 4] for the (2,4) scheme."""
        self.order = order

    def calc_derivative(self, l, k, d, n, order_of_derivative):
        """Staggered FD approximation of accuracy n (fields.py:64-69)."""
        return Deriv_half(self, l, k, d, n // 2)[order_of_derivative]

    def populate_derivatives(self, max_order=1):
        """Fill ``self.d[index][order]`` with DDerivative objects carrying FD
        approximations of every even accuracy up to the field's order
        (fields.py:71-96)."""
        self.d = [[None] * (max_order + 1) for _ in range(self.dimension + 1)]
        for d in range(self.dimension + 1):
            index = self.indices[d]
            for order in range(1, max_order + 1):
                name = ''.join(['\\partial ', self.label.name, '/\\partial ', str(index)])
                self.d[d][order] = DDerivative(name, index, order, self.order[d])
                for accuracy in range(2, self.order[d] + 2, 2):
                    self.d[d][order].fd[accuracy] = self.calc_derivative(
                        self.indices, d, self.spacing[d], accuracy, order)

    def align(self, expr):
        """Shift array indices in ``expr`` from this field's staggered frame
        to absolute array positions (fields.py:98-138): a field staggered
        differently along index k moves by +-1/2 there; media move by +1/2
        along every spatial axis this field is staggered on."""
        if expr.is_Symbol or expr.is_Number:
            return expr
        if isinstance(expr, Indexed):
            b = expr.base
            if not isinstance(b, (VField, SField, Media)):
                return expr
            if isinstance(b, Media):
                idx = list(expr.indices)
                for d in range(self.dimension):
                    if self.staggered[d + 1]:
                        idx[d] += hf
                return b[idx]
            idx = []
            for k in range(len(expr.indices)):
                if self.staggered[k] == b.staggered[k]:
                    idx.append(expr.indices[k])
                elif self.staggered[k]:
                    idx.append(expr.indices[k] + hf)
                else:
                    idx.append(expr.indices[k] - hf)
            return b[idx]
        args = tuple(self.align(arg) for arg in expr.args)
        return expr.func(*args)

    def set_fd_kernel(self, kernel):
        """Store the update kernel and its aligned form (fields.py:140-149)."""
        self.kernel = kernel
        self.kernel_aligned = self.align(kernel)

    def set_dt(self, dt):
        """Right-hand side of dF/dt, used by the free-surface conditions."""
        self.dt = dt

    def associate_stress_fields(self, sfields):
        """Stress fields this field's ghosts are solved from."""
        self.sfields = sfields


class VField(Field):
    """Velocity component; staggered in time and along its own direction
    (fields.py:169-190)."""

    def set(self, dimension, direction):
        self.direction = direction
        staggered = [False] * (dimension + 1)
        staggered[0] = True
        staggered[direction] = True
        Field.set(self, dimension, staggered)

    def set_free_surface(self, d, b, side, algo='robertsson'):
        """Ghost equations for a free surface normal to index d at array
        position b (fields.py:192-261).

        levander: the velocity along the normal comes from zero normal
        traction T_dd' = 0 (2nd-order FD); the tangential components from
        continuity of the shear-stress rate across the surface.
        robertsson: order/2 ghost layers set to zero."""
        if algo == 'levander':
            field = self.sfields[d]
            expr = field.dt
            idx = list(self.indices)
            subs = {}
            for deriv in get_all_objects(expr, DDerivative):
                subs[deriv] = deriv.fd[2]
            expr = expr.subs(subs)
            if self.staggered[d]:
                eq = Eq(expr, 0)
                shift = hf
                t = b - hf
            else:
                eq = Eq(expr.subs(idx[d], idx[d] - hf),
                        expr.subs(idx[d], idx[d] + hf))
                shift = 1
                t = b
            idx[d] -= ((-1) ** side) * shift
            lhs = self[idx]
            rhs = solve(eq, lhs)[0]
            lhs = lhs.subs(self.indices[d], t)
            rhs = self.align(rhs.subs(self.indices[d], t))
            lhs = lhs.subs(idx[0], idx[0] + 1)
            rhs = rhs.subs(idx[0], idx[0] + 1)
            self.bc[d][side] = [Eq(lhs, rhs)]
        elif algo == 'robertsson':
            idx = list(self.indices)
            if self.staggered[d]:
                idx[d] = b - (1 - side)
            else:
                idx[d] = b - (-1) ** side
            eq = Eq(self[idx], 0)
            eq = eq.subs(idx[0], idx[0] + 1)
            self.bc[d][side] = [eq]
            for depth in range(self.order[d] // 2 - 1):
                idx[d] -= (-1) ** side
                eq = Eq(self[idx], 0)
                eq = eq.subs(idx[0], idx[0] + 1)
                self.bc[d][side].append(eq)
        else:
            raise ValueError('Unknown boundary condition algorithm')


class SField(Field):
    """Stress component; normal stresses are unstaggered, shear stresses are
    staggered along both of their indices (fields.py:264-292)."""

    def set(self, dimension, direction):
        self.direction = direction
        staggered = [False] * (dimension + 1)
        if direction[0] != direction[1]:
            for i in range(len(direction)):
                staggered[direction[i]] = True
        Field.set(self, dimension, staggered)

    def set_free_surface(self, d, b, side, algo='robertsson'):
        """Ghost equations for a free surface normal to index d at array
        position b (fields.py:294-381).

        Stresses with d among their indices are mirrored antisymmetrically
        (T=0 on the surface).  With levander, normal stresses along the other
        axes are recomputed on the surface plane from a 2nd-order time step
        with dU_d/dx_d eliminated through T_dd = 0."""
        idx = list(self.indices)
        if d not in self.direction:
            if (algo != 'levander') or (self.direction[0] != self.direction[1]):
                self.bc[d][side] = []
                return
            expr = self.dt
            deriv_0 = deriv_sub = None
            for deriv in get_all_objects(expr, DDerivative):
                if deriv.var == idx[d]:
                    expr2 = self.sfields[d].dt
                    deriv_0 = deriv
                    deriv_sub = solve(expr2, deriv)[0]
                    break
            expr = expr.subs(deriv_0, deriv_sub)
            subs = {}
            for deriv in get_all_objects(expr, DDerivative):
                subs[deriv] = deriv.fd[4]
            expr = expr.subs(subs)
            eq = Eq(self.d[0][1].fd[2], expr)
            eq = eq.subs(idx[d], b)
            t = idx[0]
            idx[0] = t + hf
            idx[d] = b
            lhs = self[idx]
            rhs = solve(eq, lhs)[0]
            rhs = self.align(rhs)
            lhs = lhs.subs(t, t + hf)
            rhs = rhs.subs(t, t + hf)
            self.bc[d][side] = [Eq(lhs, rhs)]
            return

        idx = list(self.indices)
        idx2 = list(self.indices)
        if not self.staggered[d]:
            idx[d] = b
            idx2[d] = b
            eq1 = Eq(self[idx], 0)
        else:
            idx[d] = b - (1 - side)
            idx2[d] = idx[d] + (-1) ** side
            eq1 = Eq(self[idx], -self[idx2])
        eq1 = eq1.subs(idx[0], idx[0] + 1)
        self.bc[d][side] = [eq1]
        for depth in range(self.order[d] // 2 - 1):
            idx[d] -= (-1) ** side
            idx2[d] += (-1) ** side
            eq = Eq(self[idx], -self[idx2])
            eq = eq.subs(idx[0], idx[0] + 1)
            self.bc[d][side].append(eq)


class Media(IndexedBase):
    """Media parameter array (rho, vp, vs, lambda, mu and the effective
    averages), fields.py:384-406."""

    def __new__(cls, name, *args, **kwargs):
        label = name.name if isinstance(name, Symbol) else str(name)
        key = (cls, label)
        if not kwargs and key in _registry:
            return _registry[key]
        obj = IndexedBase.__new__(cls, label)
        if kwargs:
            _registry[key] = obj
        return obj

    def __init__(self, *args, **kwargs):
        if len(kwargs) > 0:
            self.set(**kwargs)

    def set(self, dimension, staggered, index):
        self.dimension = dimension
        self.staggered = staggered
        self.index = index


class RegularField(Field):
    """Unstaggered field of the acoustic RegularGrid scheme (fields.py:409-419)."""

    def __new__(cls, name, *args, **kwargs):
        return Field.__new__(cls, name, *args, **kwargs)

    def __init__(self, *args, **kwargs):
        kwargs.setdefault('staggered', [0, 0, 0])
        super().__init__(*args, **kwargs)

    def calc_derivative(self, l, k, d, n, order_of_derivative):
        return Deriv(self, l, k, d, n)[order_of_derivative]
