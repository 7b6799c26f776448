"""Regular grid: geometry, orders, time levels, switches and the symbolic
kernel transforms shared by all grids (restates opesci/regulargrid.py).
"""
import mmap
from sympy import Symbol, solve, expand

from .grid import Grid
from .variable import Variable
from .derivative import DDerivative
from .fields import RegularField
from .util import hf, get_all_objects, get_ops_expr, variable_to_symbol

__all__ = ['RegularGrid']


class RegularGrid(Grid):
    """Grid holding dimension, grid size, margins, spacing, time levels and
    code-generation switches (regulargrid.py:16-80)."""

    _papi_events = []
    _switches = ['omp', 'ivdep', 'simd', 'double', 'expand', 'eval_const',
                 'output_vts', 'converge', 'profiling', 'pluto', 'fission']
    _params = ['c', 'v']

    def __init__(self, dimension, index=None, fields=None, double=False,
                 profiling=False, pluto=False, fission=False, omp=True,
                 ivdep=True, simd=False, io=False, expand=True,
                 eval_const=True, grid_size=(10, 10, 10), domain_size=None,
                 output_vts=False):
        super().__init__()
        self.dimension = dimension
        self.double = double
        self.real_t = 'double' if self.double else 'float'
        self.dt = Variable('dt', 0.01, self.real_t, True)
        self.ntsteps = Variable('ntsteps', 100, 'int', True)
        self.alignment = mmap.PAGESIZE
        self.margin = Variable('margin', 2, 'int', True)
        self.dim = [Variable('dim' + str(k + 1), 10 + 1 + self.margin.value * 2, 'int', True)
                    for k in range(self.dimension)]
        self.size = [1.0] * dimension
        default_order = [2] + [4] * self.dimension
        self.t = Symbol('_t')
        self.grid_size = grid_size
        self.max_derivative_order = 1
        if fields is not None:
            self.fields = fields
        self.set_order(default_order)
        self.set_grid_size(grid_size)
        self._update_spacing()
        self.set_field_spacing()
        self.set_index(index)
        self.defined_variable = {}
        self.pluto = pluto
        self.omp = omp
        self.ivdep = ivdep
        self.simd = simd
        self.output_vts = output_vts
        self.expand = expand
        self.eval_const = eval_const
        self.profiling = profiling
        self.fission = fission
        self.converge = getattr(self, 'converge', False)
        if domain_size:
            self.set_domain_size(domain_size)
        self.read = False
        self.initialize_template()

    # ------------------------------------------------------------------ setup
    def initialize_template(self):
        """The CUDA program template of the acoustic scheme (StaggeredGrid
        overrides it with the elastic one)."""
        from .templates.regular_tmpl import RegularCudaTemplate
        self.cgen_template = RegularCudaTemplate(self)

    def set_variable(self, var, value=0, type='int', constant=False):
        """Define a named constant/variable of the generated program
        (regulargrid.py:85-95)."""
        if isinstance(var, Symbol):
            var = var.name
        self.defined_variable[var] = Variable(var, value, type, constant)

    def calc_derivatives(self, max_order=1):
        self.max_derivative_order = max_order
        self.set_order(self.order)
        for field in self.fields:
            field.populate_derivatives(max_order=max_order)

    def set_order(self, order):
        """Scheme order [time, space...]; creates time-level variables and
        sets the margin to space_order/2 (regulargrid.py:106-131)."""
        for x in order:
            if x % 2 == 1:
                raise ValueError(str(x) + ' is not a valid order (require even integer)')
        self.order = order
        num_time_vars = max(self.order[0], self.max_derivative_order + 1)
        self.tp = Variable('tp', num_time_vars, 'int', True)
        self.time = []
        for k in range(num_time_vars):
            self.time.append(Variable(str(self.t) + str(k), k, 'int', False))
        self.margin.value = self.order[1] // 2
        self.set_grid_size(self.grid_size)
        self.update_field_order()
        self._update_spacing()

    def get_time_step_limit(self):
        h = min([sp.value for sp in self.spacing])
        return h / (3 ** 0.5 * self.c)

    def set_domain_size(self, size):
        self.size = size
        self._update_spacing()

    def set_grid_size(self, size):
        """dimK = n_K + 1 + 2*margin (regulargrid.py:145-155)."""
        self.grid_size = size
        self.dim = [Variable('dim' + str(k + 1), size[k] + 1 + 2 * self.margin.value, 'int', True)
                    for k in range(self.dimension)]
        self._update_spacing()

    def update_field_order(self):
        if hasattr(self, 'fields'):
            for field in self.fields:
                field.set_order(self.order)

    def set_time_step(self, dt, tmax):
        """dt and ntsteps = int(tmax/dt) (regulargrid.py:165-172)."""
        self.dt.value = dt
        self.ntsteps.value = int(tmax / dt)

    def set_switches(self, **kwargs):
        """Boolean code-generation switches (regulargrid.py:174-185)."""
        for switch, value in kwargs.items():
            if switch not in self._switches:
                raise KeyError("Unsupported switch: ", switch)
            if not isinstance(value, bool):
                raise ValueError("Only boolean values allowed for switches")
            setattr(self, switch, value)
            if switch == 'double':
                self.real_t = 'double' if self.double else 'float'
                self._update_spacing()
        self.initialize_template()

    def _update_spacing(self):
        """dxK = size_K / (dimK - 1 - 2*margin) (regulargrid.py:187-201)."""
        self.spacing = [Variable('dx' + str(k + 1),
                                 self.size[k] / (self.dim[k].value - 1 - self.margin.value * 2),
                                 self.real_t, True) for k in range(self.dimension)]
        expr = self.order[0]
        for d in self.dim:
            expr *= d
        self.vec_size = Variable('vec_size', expr, 'int', True)

    def set_index(self, index):
        if index is None:
            self.index = [Symbol('x' + str(k + 1)) for k in range(self.dimension)]
        else:
            self.index = index
        if hasattr(self, 'fields'):
            for field in self.fields:
                field.set_indices([self.t] + self.index)

    def set_params(self, **kwargs):
        for param, value in kwargs.items():
            if param not in self._params:
                raise KeyError("Unsupported parameter: ", param)
            setattr(self, param, value)
            self.set_variable(param, value, self.real_t, True)

    def set_field_spacing(self):
        for field in self.fields:
            field.set_spacing(variable_to_symbol([self.dt] + self.spacing))

    # ------------------------------------------------------- symbolic solve
    def solve_fd(self, equations):
        """Solve each PDE for the most advanced time level
        (regulargrid.py:230-270)."""
        self.eq = []
        if len(self.fields) != len(equations):
            raise KeyError("Number of equations must be the same as number of fields. "
                           "Number of fields is ", len(self.fields))
        for field, eq in zip(self.fields, equations):
            field.set_dt(eq.rhs)
            self.eq.append(eq)
        eqs = []
        for eq in self.eq:
            for deriv in get_all_objects(eq, DDerivative):
                eq = eq.subs(deriv, deriv.fd[deriv.max_accuracy])
            eqs.append(eq)
        t = self.t
        t1 = t + hf + (self.order[0] // 2 - 1)
        t1_regular = t + 1 + (self.order[0] // 2 - 1)
        index = [t1] + self.index
        index_regular = [t1_regular] + self.index
        simplify = max(self.order[1:]) <= 4
        for field, eq in zip(self.fields, eqs):
            if isinstance(field, RegularField):
                kernel = solve(eq, field[index_regular], simplify=simplify)[0]
            else:
                kernel = solve(eq, field[index], simplify=simplify)[0]
            kernel = kernel.subs({t: t - (self.order[0] // 2 - 1)})
            field.set_fd_kernel(kernel)

    def get_all_variables(self):
        return (self.dim + self.spacing + self.time
                + [self.tp, self.dt, self.margin, self.ntsteps]
                + list(self.defined_variable.values()))

    def create_const_dict(self):
        """Values of every constant, folded into kernels when eval_const is
        set (regulargrid.py:281-291)."""
        consts = {}
        for v in self.get_all_variables():
            if v.constant:
                consts[Symbol(v.name)] = v.value
        self.const_dict = consts

    def get_kernel_ai(self, fields=None):
        """(AI, weighted AI, #ADD, #MUL, #LOAD, #STORE) of the update kernels
        of ``fields`` (regulargrid.py:293-327)."""
        if fields is None:
            fields = self.fields
        if self.eval_const:
            self.create_const_dict()
        store = add = mul = 0
        arrays = []
        for field in fields:
            store += 1
            expr = self.transform_kernel(field)
            add2, mul2, arrays = get_ops_expr(expr, arrays)
            add += add2
            mul += mul2
        word_size = 8 if self.double else 4
        load = len(arrays)
        ai = float(add + mul) / (load + store) / word_size
        ai_w = ai * (add + mul) / max(add, mul) / 2.0
        return (ai, ai_w, add, mul, load, store)

    def transform_kernel(self, field):
        """Expand and constant-fold a kernel (regulargrid.py:329-342)."""
        kernel_new = field.kernel_aligned
        if self.expand:
            kernel_new = expand(kernel_new)
        if self.eval_const:
            kernel_new = kernel_new.subs(self.const_dict)
        return kernel_new

    def kernel_sympy(self, field):
        """Transformed kernel with t+1 -> t2, t -> t1, t-1 -> t0
        (regulargrid.py:592-595)."""
        if self.eval_const:
            self.create_const_dict()
        kernel = self.transform_kernel(field)
        return kernel.xreplace({self.t + 1: self.time[2], self.t: self.time[1], self.t - 1: self.time[0]})

    def initial_kernel(self, field):
        """Right-hand side of the first initialisation, level 0 on the whole
        padded grid (regulargrid.py:498-534): the analytic solution at t = 0
        with the loop indices _x, _y, _z substituted for the coordinates, as
        the reference does."""
        sol = field.sol.subs(self.t, 0)
        for idx in self.index:
            sol = sol.subs(idx, '_' + idx.name)
        return sol

    def second_initial_kernel(self, field):
        """Right-hand side of the second initialisation, level _t1 on the
        interior (regulargrid.py:536-564): the update kernel with its
        negative t-1 term dropped, halved, plus v*dt, read at level _t0."""
        v = Symbol('v')
        if self.eval_const:
            self.create_const_dict()
        kernel = self.transform_kernel(field)
        for arg in kernel.args:
            if str(arg).startswith('-') and str(self.t - 1) in str(arg):
                kernel = kernel.subs({arg: 0}, simultaneous=True)
                arg = 2 * v * self.dt
                kernel = 0.5 * (kernel + arg)
        kernel = kernel.subs({self.t: self.time[0]})
        for idx in self.index:
            kernel = kernel.subs(idx, '_' + idx.name)
        return kernel

    def set_papi_events(self, events=[]):
        self._papi_events = events

    @property
    def numevents_papi(self):
        return len(self._papi_events)

    @property
    def io(self):
        return self.output_vts
