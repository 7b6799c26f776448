"""Model builders: the 3D elastic eigenmode problem, seeded layered media and
Ricker wavelets.

``eigenwave_grid`` builds, through the public StaggeredGrid API, the same
model as the reference's model script tests/eigenwave3d.py:9-146: nine fields,
the velocity-stress PDEs, the standing-wave eigenmode as initial condition and
analytic solution, and free surfaces on all six faces.  The physics has to be
identical for parity, so the field definitions, PDEs and analytic functions
are the reference's; the code around them is this package's.
"""
import math

import numpy as np
from sympy import symbols, Eq, sqrt, pi, cos, sin, Float

from .fields import SField, VField
from .staggeredgrid import StaggeredGrid
from .util import staggered_weights

__all__ = ['eigenwave_grid', 'elastic_grid', 'layered_media', 'ricker',
           'stable_dt', 'cfl_dt', 'simplewave_grid']


def _elastic_fields():
    Txx = SField('Txx', dimension=3, direction=(1, 1))
    Tyy = SField('Tyy', dimension=3, direction=(2, 2))
    Tzz = SField('Tzz', dimension=3, direction=(3, 3))
    Txy = SField('Txy', dimension=3, direction=(1, 2))
    Tyz = SField('Tyz', dimension=3, direction=(2, 3))
    Txz = SField('Txz', dimension=3, direction=(1, 3))
    U = VField('U', dimension=3, direction=1)
    V = VField('V', dimension=3, direction=2)
    W = VField('W', dimension=3, direction=3)
    return (Txx, Tyy, Tzz, Txy, Tyz, Txz), (U, V, W)


def elastic_grid(domain_size, grid_size, dt, tmax, space_order=4, read=False,
                 rho=1.0, vp=1.0, vs=0.5, rho_file='', vp_file='', vs_file='',
                 analytic=True, free_surface=True, double=False,
                 expand=True, eval_const=True, media_override=None):
    """Build and solve the elastic velocity-stress model.

    With ``analytic`` the eigenmode of tests/eigenwave3d.py:88-108 is set as
    initial condition/analytic solution; otherwise fields start at zero.
    ``media_override`` replaces the constant (rho, beta, lambda, mu) values
    after set_media_params (used to pin the older generator's constants)."""
    (Txx, Tyy, Tzz, Txy, Tyz, Txz), (U, V, W) = _elastic_fields()
    grid = StaggeredGrid(dimension=3, domain_size=domain_size, grid_size=grid_size,
                         stress_fields=[Txx, Tyy, Tzz, Txy, Tyz, Txz],
                         velocity_fields=[U, V, W])
    grid.set_time_step(dt, tmax)
    grid.set_switches(double=double, expand=expand, eval_const=eval_const,
                      converge=bool(analytic))
    rho_s, beta, lam, mu = symbols('rho beta lambda mu')
    t, x, y, z = symbols('_t x y z')
    grid.set_index([x, y, z])
    if read:
        grid.set_media_params(read=True, rho_file=rho_file, vp_file=vp_file, vs_file=vs_file)
    else:
        grid.set_media_params(read=False, rho=rho, vp=vp, vs=vs)
        if media_override:
            for k, v in media_override.items():
                grid.defined_variable[k].value = v
    if analytic:
        Omega = pi * sqrt(2 * mu * beta)
        A = sqrt(2 * mu / beta)
        U.set_analytic_solution(cos(pi * x) * (sin(pi * y) - sin(pi * z)) * cos(Omega * t))
        V.set_analytic_solution(cos(pi * y) * (sin(pi * z) - sin(pi * x)) * cos(Omega * t))
        W.set_analytic_solution(cos(pi * z) * (sin(pi * x) - sin(pi * y)) * cos(Omega * t))
        Txx.set_analytic_solution(-A * sin(pi * x) * (sin(pi * y) - sin(pi * z)) * sin(Omega * t))
        Tyy.set_analytic_solution(-A * sin(pi * y) * (sin(pi * z) - sin(pi * x)) * sin(Omega * t))
        Tzz.set_analytic_solution(-A * sin(pi * z) * (sin(pi * x) - sin(pi * y)) * sin(Omega * t))
        for f in (Txy, Tyz, Txz):
            f.set_analytic_solution(Float(0))
    else:
        for f in grid.fields:
            f.sol = None
    grid.set_order([2, space_order, space_order, space_order])
    grid.calc_derivatives()
    eqs = [
        Eq(U.d[0][1], beta * (Txx.d[1][1] + Txy.d[2][1] + Txz.d[3][1])),
        Eq(V.d[0][1], beta * (Txy.d[1][1] + Tyy.d[2][1] + Tyz.d[3][1])),
        Eq(W.d[0][1], beta * (Txz.d[1][1] + Tyz.d[2][1] + Tzz.d[3][1])),
        Eq(Txx.d[0][1], (lam + 2 * mu) * U.d[1][1] + lam * (V.d[2][1] + W.d[3][1])),
        Eq(Tyy.d[0][1], (lam + 2 * mu) * V.d[2][1] + lam * (U.d[1][1] + W.d[3][1])),
        Eq(Tzz.d[0][1], (lam + 2 * mu) * W.d[3][1] + lam * (U.d[1][1] + V.d[2][1])),
        Eq(Txy.d[0][1], mu * (U.d[2][1] + V.d[1][1])),
        Eq(Tyz.d[0][1], mu * (V.d[3][1] + W.d[2][1])),
        Eq(Txz.d[0][1], mu * (U.d[3][1] + W.d[1][1])),
    ]
    grid.solve_fd(eqs)
    if free_surface:
        for dim in (1, 2, 3):
            for side in (0, 1):
                grid.set_free_surface_boundary(dimension=dim, side=side)
    return grid


def eigenwave_grid(grid_size=(64, 64, 64), dt=None, ntsteps=200, space_order=4,
                   legacy=False, **kw):
    """The eigenwave problem on the unit cube.  ``dt`` defaults to half the
    stable step of the scheme (``cfl_dt``).  ``legacy`` reproduces the older
    generator behind benchmarks/test3d.cpp (lambda = mu = 0.5, no
    normal-stress recompute on the free surfaces)."""
    h = 1.0 / grid_size[0]
    if dt is None:
        dt = cfl_dt(h, 1.0, space_order)
    tmax = dt * ntsteps
    override = {'rho': 1.0, 'beta': 1.0, 'lambda': 0.5, 'mu': 0.5} if legacy else None
    grid = elastic_grid((1.0, 1.0, 1.0), grid_size, dt, tmax, space_order=space_order,
                        media_override=override, **kw)
    # int(tmax/dt) may round down by one for some dt; pin the step count
    grid.ntsteps.value = ntsteps
    grid.legacy_bc = legacy
    return grid


def simplewave_grid(domain_size=(1.0, 1.0, 1.0), grid_size=(100, 100, 100), dt=0.002, tmax=1.0,
                    space_order=4, double=False, ntsteps=None):
    """The acoustic model of tests/simplewaveequation.py:9-81, built through
    the public RegularGrid API: one RegularField, c = 2 and v = 1, the
    analytic function -A sin(pi x)(sin(pi y) - sin(pi z)) sin(Omega t) with
    mu = 10, beta = 0.5, and the model's equation as written there,
    u_tt = c^2 (u_xx + u_yy + u_yy).  ``ntsteps`` overrides int(tmax/dt)."""
    from .fields import RegularField
    from .regulargrid import RegularGrid
    main = RegularField('MAIN_GRID', dimension=3)
    grid = RegularGrid(dimension=3, domain_size=domain_size, grid_size=grid_size, fields=[main])
    grid.set_time_step(dt, tmax)
    if ntsteps is not None:
        grid.ntsteps.value = int(ntsteps)
    grid.set_switches(double=double, expand=True, eval_const=True, converge=True)
    t, x, y, z, c = symbols('_t x y z c')
    grid.set_index([x, y, z])
    grid.set_params(c=2, v=1)
    mu, beta = 10, 0.5
    Omega = pi * sqrt(2 * mu * beta)
    A = sqrt(2 * mu / beta)
    main.set_analytic_solution(-A * sin(pi * x) * (sin(pi * y) - sin(pi * z)) * sin(Omega * t))
    grid.set_order([2, space_order, space_order, space_order])
    grid.calc_derivatives(2)
    grid.solve_fd([Eq(main.d[0][2], (c ** 2) * (main.d[1][2] + main.d[2][2] + main.d[2][2]))])
    return grid


def stable_dt(h, vmax, space_order):
    """Stability limit h / (sqrt(3) vmax sum|c_k|) of the staggered leapfrog
    scheme; for space order 4 this is 6/7 h/(sqrt(3) vmax) = 0.4949 h/vmax,
    the 0.495 h/Vp of staggeredgrid.py:99-100 and opesciHandy.cpp:69-89."""
    s = sum(abs(float(c)) for c in staggered_weights(space_order))
    return h / (math.sqrt(3.0) * vmax * s)


def cfl_dt(h, vmax, space_order, cfl=0.5):
    """``cfl`` times the stable step (the time step convention of this
    package's benchmark configurations)."""
    return cfl * stable_dt(h, vmax, space_order)


def ricker(nt, dt, f0):
    """Ricker wavelet r(t) = (1 - 2 pi^2 f^2 (t-t0)^2) exp(-pi^2 f^2 (t-t0)^2)
    with t0 = 1/f, sampled at t = i*dt, float32."""
    t = np.arange(nt, dtype=np.float64) * dt - 1.0 / f0
    a = (np.pi * f0 * t) ** 2
    return ((1.0 - 2.0 * a) * np.exp(-a)).astype(np.float32)


def _smooth_axis(a, radius, axis):
    # three passes of a box filter of width 2r+1 approximate a Gaussian
    from scipy.ndimage import uniform_filter1d
    for _ in range(3):
        a = uniform_filter1d(a, size=2 * radius + 1, axis=axis, mode='nearest')
    return a


def layered_media(dims, seed=0, nlayers=20, vp_range=(1500.0, 4500.0), perturb=0.05,
                  radius=3, depth_axis=2):
    """Seeded layered elastic medium on an array of shape ``dims`` (margins
    included, reference layout [dim1][dim2][dim3], z contiguous).

    ``nlayers`` equal layers along ``depth_axis`` with vp ~ U(vp_range) m/s,
    times (1 + perturb * n) where n is N(0,1) noise smoothed by a
    Gaussian-like filter and renormalised to unit variance; vs = vp/sqrt(3);
    density from Gardner's rule rho = 310 vp^0.25 kg/m^3 (0.31 vp^0.25 g/cc).
    Returns float32 (rho, vp, vs)."""
    rng = np.random.default_rng(seed)
    layer_vp = rng.uniform(vp_range[0], vp_range[1], size=nlayers)
    n = dims[depth_axis]
    layer_of = np.minimum((np.arange(n) * nlayers) // n, nlayers - 1)
    prof = layer_vp[layer_of].astype(np.float32)
    shape = [1, 1, 1]
    shape[depth_axis] = n
    noise = rng.standard_normal(size=tuple(dims), dtype=np.float32)
    for ax in range(3):
        noise = _smooth_axis(noise, radius, ax)
    noise /= max(float(noise.std()), 1e-12)
    vp = (prof.reshape(shape) * (1.0 + perturb * noise)).astype(np.float32)
    vs = (vp / np.float32(math.sqrt(3.0))).astype(np.float32)
    rho = (np.float32(310.0) * np.power(vp, np.float32(0.25))).astype(np.float32)
    return rho, vp, vs


def _field_ranges(grid, field):
    """Index range and coordinates per axis of a field's own points:
    [m, dim-m) unstaggered, [m, dim-m-1) staggered, coordinate
    h*(i-m) or h*(i-m+1/2) rounded to the grid's real type like the
    generated code's ``real_t x = dx1*(_x - m)`` (staggeredgrid.py:632-641)."""
    m = grid.margin.value
    real = np.float64 if grid.double else np.float32
    out = []
    for d in range(grid.dimension):
        hi = grid.dim[d].value - m - (1 if field.staggered[d + 1] else 0)
        idx = np.arange(m, hi)
        h = real(grid.spacing[d].value)
        off = 0.5 if field.staggered[d + 1] else 0.0
        coord = (np.float64(h) * (idx - m + off)).astype(real)
        out.append((m, hi, coord.astype(np.float64)))
    return out


def _sol_function(grid, field):
    import sympy
    consts = {}
    real = np.float64 if grid.double else np.float32
    for v in grid.defined_variable.values():
        consts[sympy.Symbol(v.name)] = float(real(v.value))
    sol = field.sol
    syms = [grid.t] + list(grid.index)
    expr = sympy.sympify(sol).subs(consts)
    return sympy.lambdify(syms, expr, modules='numpy')


def analytic_field(grid, field, t):
    """The field's analytic solution at time t on its own index range
    (zero elsewhere), in the reference layout, as the grid's real type."""
    real = np.float64 if grid.double else np.float32
    dims = tuple(d.value for d in grid.dim)
    out = np.zeros(dims, dtype=real)
    if getattr(field, 'sol', None) is None:
        return out
    (x0, x1, cx), (y0, y1, cy), (z0, z1, cz) = _field_ranges(grid, field)
    f = _sol_function(grid, field)
    X, Y, Z = np.meshgrid(cx, cy, cz, indexing='ij')
    val = f(float(t), X, Y, Z)
    out[x0:x1, y0:y1, z0:z1] = np.broadcast_to(np.asarray(val, dtype=np.float64), X.shape).astype(real)
    return out


def initial_fields(grid):
    """Initial level of every field: stresses at t=0, velocities at t=dt/2
    (staggeredgrid.py:647)."""
    out = {}
    for f in grid.fields:
        t0 = grid.dt.value / 2 if f.staggered[0] else 0.0
        out[f.label.name] = analytic_field(grid, f, t0)
    return out


def l2_error(grid, field, values):
    """FP64 L2 error sqrt(sum (f - f_exact(t_end))^2 * dx1 dx2 dx3) of a final
    field over its own index range, t_end = dt*ntsteps (+dt/2 for velocities),
    the norm of staggeredgrid.py:892-945 with an FP64 accumulator."""
    (x0, x1, cx), (y0, y1, cy), (z0, z1, cz) = _field_ranges(grid, field)
    tn = grid.dt.value * grid.ntsteps.value + (grid.dt.value / 2.0 if field.staggered[0] else 0.0)
    f = _sol_function(grid, field)
    X, Y, Z = np.meshgrid(cx, cy, cz, indexing='ij')
    exact = np.broadcast_to(np.asarray(f(float(tn), X, Y, Z), dtype=np.float64), X.shape)
    diff = values[x0:x1, y0:y1, z0:z1].astype(np.float64) - exact
    vol = 1.0
    for sp in grid.spacing:
        vol *= sp.value
    return float(np.sqrt(np.sum(diff * diff) * vol))


def layered_problem(n, space_order=4, ntsteps=100, h=10.0, seed=0, f0=15.0, media_files=None,
                    cfl=0.5, free_surface=True):
    """The at-scale forward-modelling problem on an n^3 interior grid:
    seeded layered media (``layered_media``), spacing ``h`` metres, a Ricker
    source of peak frequency ``f0`` injected into the normal stresses at a
    seeded interior point, dt = ``cfl`` x the stable step for the fastest vp.

    The grid is built in read mode (media from raw files, effective-media
    averaging of staggeredgrid.py:522-598).  ``media_files`` (dict with keys
    rho, vp, vs) are written when given, for programs that read the files.
    Returns (grid, (rho, vp, vs), source_index, wavelet)."""
    m = space_order // 2
    dims = (n + 2 * m,) * 3
    rho, vp, vs = layered_media(dims, seed=seed)
    vmax = float(vp.max())
    dt = cfl_dt(h, vmax, space_order, cfl=cfl)
    files = media_files or {'rho': '', 'vp': '', 'vs': ''}
    if media_files:
        for k, a in (('rho', rho), ('vp', vp), ('vs', vs)):
            a.tofile(media_files[k])
    grid = elastic_grid((h * (n - 1),) * 3, (n - 1,) * 3, dt, dt * ntsteps, space_order=space_order,
                        read=True, rho_file=files['rho'], vp_file=files['vp'], vs_file=files['vs'],
                        analytic=False, free_surface=free_surface)
    grid.ntsteps.value = ntsteps
    rng = np.random.default_rng(seed + 7919)
    src = tuple(int(v) for v in rng.integers(m + n // 4, m + 3 * n // 4, size=3))
    wav = ricker(ntsteps, dt, f0)
    return grid, (rho, vp, vs), src, wav
