"""StaggeredGrid: the velocity-stress elastic scheme on a staggered grid.

Restates the symbolic side of opesci/staggeredgrid.py (reference): field
registration, time-step limit, stencil substitution and solve, free-surface
conditions, media parameters (constant or read from raw files with
effective-media averaging) and the arithmetic-intensity counters.  The time
loop itself runs in the CUDA device runtime (libofd), driven by the CUDA
program template in opesci/templates/cuda_tmpl.py.
"""
from sympy import Symbol, Rational, solve, expand, Eq, Indexed
from sympy.core.cache import clear_cache

from .fields import Media, SField, VField
from .derivative import DDerivative
from .util import get_all_objects, get_ops_expr, is_half, staggered_weights
from .regulargrid import RegularGrid

__all__ = ['StaggeredGrid']

hf = Rational(1, 2)


class StaggeredGrid(RegularGrid):
    """Velocity-stress scheme on a staggered grid (staggeredgrid.py:15-67).

    Usage follows the reference: create the grid with its stress and velocity
    fields, set time step, switches, index symbols and media, set analytic
    solutions, ``set_order`` and ``calc_derivatives``, ``solve_fd`` with the
    nine PDEs, then ``set_free_surface_boundary`` for each face.  The grid is
    then generated/compiled/executed through the CUDA target.

    Switches: omp, ivdep, simd (accepted for compatibility, meaningless on the
    GPU), double (FP64 storage and arithmetic), expand, eval_const,
    output_vts, converge, profiling, pluto, fission."""

    _switches = ['omp', 'ivdep', 'simd', 'double', 'expand', 'eval_const',
                 'output_vts', 'converge', 'profiling', 'pluto', 'fission']
    _papi_events = []

    def __init__(self, stress_fields=None, velocity_fields=None, converge=False, **kwargs):
        clear_cache()
        self.sfields = []
        self.vfields = []
        self.storage = None
        self.legacy_bc = False
        super().__init__(**kwargs)
        self.converge = converge
        self.source = None
        if stress_fields:
            self.set_stress_fields(stress_fields)
        if velocity_fields:
            self.set_velocity_fields(velocity_fields)

    def initialize_template(self):
        from .templates.cuda_tmpl import StaggeredCudaTemplate
        self.cgen_template = StaggeredCudaTemplate(self)

    @property
    def fields(self):
        """Velocity fields then stress fields: the order of the OpesciGrid
        struct (staggeredgrid.py:69-71)."""
        return self.vfields + self.sfields

    @property
    def io(self):
        return self.read or self.output_vts

    def set_alignment(self, alignment):
        self.alignment = alignment

    def get_time_step_limit(self):
        """Stability limit (staggeredgrid.py:85-102): SO2 h/Vp/sqrt(3),
        SO4 0.495 h/Vp."""
        if self.read:
            return ('physical parameters to be read from file,'
                    ' please compile and run the executable')
        l = self.defined_variable['lambda'].value
        m = self.defined_variable['mu'].value
        r = self.defined_variable['rho'].value
        Vp = ((l + 2 * m) / r) ** 0.5
        h = min([sp.value for sp in self.spacing])
        if self.order[1] == 2:
            return h / Vp / (3 ** 0.5)
        elif self.order[1] == 4:
            return 0.495 * h / Vp
        return 'not implemented yet'

    def set_stress_fields(self, sfields):
        num = self.dimension + self.dimension * (self.dimension - 1) // 2
        if len(sfields) != num:
            raise Exception('wrong number of stress fields: ' + str(num) + ' fields required.')
        self.sfields = sfields
        self.set_field_spacing()

    def set_velocity_fields(self, vfields):
        num = self.dimension
        if len(vfields) != num:
            raise Exception('wrong number of velocity fields: ' + str(num) + ' fields required.')
        self.vfields = vfields
        self.set_field_spacing()

    def calc_derivatives(self):
        for field in self.sfields + self.vfields:
            field.populate_derivatives(max_order=1)

    def solve_fd(self, equations):
        """Substitute the highest-accuracy stencils into the PDEs and solve
        each for its field at t+1/2 (staggeredgrid.py:135-170)."""
        self.eq = []
        for field, eq in zip(self.fields, equations):
            if self.read:
                eq = eq.subs(self.media_dict)
            field.set_dt(eq.rhs)
            self.eq.append(eq)
        eqs = []
        for eq in self.eq:
            for deriv in get_all_objects(eq, DDerivative):
                eq = eq.subs(deriv, deriv.fd[deriv.max_accuracy])
            eqs.append(eq)
        t = self.t
        t1 = t + hf + (self.order[0] // 2 - 1)
        index = [t1] + self.index
        simplify = max(self.order[1:]) <= 4
        for field, eq in zip(self.fields, eqs):
            kernel = solve(eq, field[index], simplify=simplify)[0]
            kernel = kernel.subs({t: t + hf - (self.order[0] // 2 - 1)})
            field.set_fd_kernel(kernel)

    def transform_bc(self, field, dimension, side):
        """Expanded / constant-folded ghost equations (staggeredgrid.py:172-188)."""
        out = []
        for bc in field.bc[dimension][side]:
            bc_new = bc
            if self.expand:
                bc_new = expand(bc_new)
            if self.eval_const:
                bc_new = bc_new.subs(self.const_dict)
            out.append(bc_new)
        return out

    def associate_fields(self):
        """Pair each velocity with its stresses and each normal stress with
        the normal stresses (staggeredgrid.py:190-212)."""
        for v in self.vfields:
            fields = [None]
            for d in range(1, self.dimension + 1):
                lookfor = tuple(sorted([v.direction, d]))
                fields.append([f for f in self.sfields if f.direction == lookfor][0])
            if len(fields) != self.dimension + 1:
                raise Exception('error in field directions')
            v.associate_stress_fields(fields)
        fields = [None] + [f for f in self.sfields if f.direction[0] == f.direction[1]]
        for s in fields[1:]:
            s.associate_stress_fields(fields)

    def set_free_surface_boundary(self, dimension, side):
        """Free surface on face (dimension, side); Levander for 4th-order,
        Robertsson otherwise (staggeredgrid.py:214-232)."""
        algo = 'levander' if self.order[dimension] == 4 else 'robertsson'
        self.associate_fields()
        if not hasattr(self, 'free_surface'):
            self.free_surface = {}
        self.free_surface[(dimension, side)] = algo
        for field in self.sfields + self.vfields:
            if side == 0:
                field.set_free_surface(dimension, self.margin.value, side, algo=algo)
            else:
                field.set_free_surface(dimension, self.dim[dimension - 1].value - self.margin.value - 1,
                                       side, algo=algo)

    def set_media_params(self, read=False, rho=1.0, vp=1.0, vs=0.5,
                         rho_file='', vp_file='', vs_file=''):
        """Constant media (beta=1/rho, lambda=rho(vp^2-2vs^2), mu=rho vs^2)
        or raw-file media with effective averages (staggeredgrid.py:234-291)."""
        self.read = read
        if self.read:
            self.rho_file = rho_file
            self.vp_file = vp_file
            self.vs_file = vs_file
            kw = dict(dimension=3, staggered=[False, False, False], index=self.index)
            self.rho = Media('rho', **kw)
            self.vp = Media('vp', **kw)
            self.vs = Media('vs', **kw)
            self.beta = [Media('beta', **kw), Media('beta1', **kw),
                         Media('beta2', **kw), Media('beta3', **kw)]
            self.lam = Media('lambda', **kw)
            self.mu = [Media('mu', **kw), Media('mu12', **kw),
                       Media('mu13', **kw), Media('mu23', **kw)]
            self.create_media_dict()
        else:
            self.set_variable('rho', rho, 'float', True)
            self.set_variable('beta', 1.0 / rho, 'float', True)
            self.set_variable('lambda', rho * (vp ** 2 - 2 * vs ** 2), 'float', True)
            self.set_variable('mu', rho * (vs ** 2), 'float', True)

    def create_media_dict(self):
        self.media_dict = {Symbol('beta'): self.beta[0][self.index],
                           Symbol('lambda'): self.lam[self.index],
                           Symbol('mu'): self.mu[0][self.index]}

    def resolve_individual_media_param(self, expr):
        """Map a media parameter at a staggered position to the effective
        array at the integer position (staggeredgrid.py:293-331)."""
        idx = list(expr.indices)
        if str(expr.base.label) == 'beta':
            for k in range(3):
                if is_half(idx[k]):
                    idx[k] -= hf
                    return self.beta[k + 1][idx]
            return expr
        if str(expr.base.label) == 'mu':
            if is_half(idx[0]):
                idx[0] -= hf
                if is_half(idx[1]):
                    idx[1] -= hf
                    return self.mu[1][idx]
                idx[2] -= hf
                return self.mu[2][idx]
            elif is_half(idx[1]):
                idx[1] -= hf
                idx[2] -= hf
                return self.mu[3][idx]
            return expr
        return expr

    def resolve_media_params(self, expr):
        """Replace staggered media references by effective media arrays
        (staggeredgrid.py:333-352)."""
        if expr.is_Equality:
            return Eq(expr.lhs, self.resolve_media_params(expr.rhs))
        if expr.is_Symbol or expr.is_Number:
            return expr
        if isinstance(expr, Indexed):
            if not isinstance(expr.base, Media):
                return expr
            return self.resolve_individual_media_param(expr)
        args = tuple(self.resolve_media_params(arg) for arg in expr.args)
        return expr.func(*args)

    def kernel_sympy(self, field):
        """Transformed kernel with t+1 -> t1 and t -> t0 (staggeredgrid.py:354-359)."""
        kernel = self.transform_kernel(field)
        if self.read:
            kernel = self.resolve_media_params(kernel)
        return kernel.xreplace({self.t + 1: self.time[1], self.t: self.time[0]})

    # --------------------------------------------------- arithmetic intensity
    def get_velocity_kernel_ai(self):
        return self.get_kernel_ai(self.vfields)

    def get_stress_kernel_ai(self):
        return self.get_kernel_ai(self.sfields)

    def _bc_ai(self, fields):
        result = []
        if self.eval_const:
            self.create_const_dict()
        word_size = 8 if self.double else 4
        for field in fields:
            for dimension in range(1, 4):
                for side in range(2):
                    store = add = mul = 0
                    arrays = []
                    for bc in self.transform_bc(field, dimension, side):
                        store += 1
                        add2, mul2, arrays = get_ops_expr(bc.rhs, arrays)
                        add += add2
                        mul += mul2
                    load = len(arrays)
                    ai_w = 0
                    if store == 0:
                        ai = 0
                        weight = 0
                    else:
                        ai = float(add + mul) / (load + store) / word_size
                        weight = 1.0 / (self.dim[dimension - 1].value - self.margin.value * 2)
                        if add == 0 and mul == 0:
                            ai_w = ai
                        else:
                            ai_w = ai * (add + mul) / max(add, mul) / 2.0
                    result.append({'weight': weight, 'ai': ai, 'ai_w': ai_w, 'add': add,
                                   'mul': mul, 'load': load, 'store': store})
        return result

    def get_velocity_bc_ai(self):
        """Per-face AI of the velocity ghost updates (staggeredgrid.py:385-431)."""
        return self._bc_ai(self.vfields)

    def get_stress_bc_ai(self):
        """Per-face AI of the stress ghost updates (staggeredgrid.py:433-479)."""
        return self._bc_ai(self.sfields)

    def get_overall_kernel_ai(self):
        """Weighted AI of kernels and boundaries with ghost adjustment
        (staggeredgrid.py:481-510)."""
        velocity_ai = self.get_velocity_kernel_ai()
        stress_ai = self.get_stress_kernel_ai()
        total_weight = 2.0
        overall_ai = velocity_ai[0] + stress_ai[0]
        overall_ai_w = velocity_ai[1] + stress_ai[1]
        for ai in self.get_velocity_bc_ai() + self.get_stress_bc_ai():
            total_weight += ai['weight']
            overall_ai += ai['ai'] * ai['weight']
            overall_ai_w += ai['ai_w'] * ai['weight']
        overall_ai /= total_weight
        overall_ai_w /= total_weight
        ghost_adj = 1.0
        for d in self.dim[1:]:
            ghost_adj *= 1 - float(self.margin.value) / d.value
        return overall_ai * ghost_adj, overall_ai_w * ghost_adj

    # ------------------------------------------------- device-runtime inputs
    def space_order(self):
        return self.order[1]

    def fd_weights(self):
        """Staggered first-derivative weights c_1..c_R of the scheme's spatial
        accuracy, as floats (from the same Taylor inverse as the kernels)."""
        return [float(w) for w in staggered_weights(self.order[1])]

    def set_source(self, position, wavelet):
        """Point source injected as T_ii[src] -= s_i(t)/3 into the three normal
        stresses after each step, following the hand-written reference solver
        (tests/src/test_ref_iso_elastic.cpp:100-126,274-290).  ``position`` is
        an array index triple (margins included); ``wavelet`` one value per
        step for all three stresses, or three such signals (x, y, z) of one
        length."""
        w = list(wavelet)
        if w and hasattr(w[0], '__len__'):
            if len(w) != 3 or len({len(s) for s in w}) != 1:
                raise ValueError('three source signals (x, y, z) of one length expected')
            w = tuple([float(v) for v in s] for s in w)
        else:
            w = [float(v) for v in w]
        self.source = (tuple(int(p) for p in position), w)
