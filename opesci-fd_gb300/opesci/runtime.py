"""ctypes binding of the device runtime libofd.so (include/ofd.h).

``Simulation`` owns one device handle: nine fields (two time levels) and the
effective media resident in HBM, advanced with ``step``.  There is no CPU
path: if the library is missing or no GPU is visible the calls raise."""
import ctypes
import os

import numpy as np

from . import build as _build

__all__ = ['OFDError', 'load_library', 'Simulation', 'FIELDS', 'STORAGE', 'BC',
           'config_from_grid', 'library_path', 'RegularSimulation', 'regular_config',
           'regular_config_from_grid']

FIELDS = ['U', 'V', 'W', 'Txx', 'Tyy', 'Tzz', 'Txy', 'Tyz', 'Txz']
STORAGE = {'f32': 0, 'float': 0, 'fp32': 0, 'f16': 1, 'fp16': 1, 'half': 1,
           'bf16': 2, 'bfloat16': 2, 'f64': 3, 'double': 3, 'fp64': 3}
BC = {'none': 0, 'levander': 1, 'robertsson': 2}


class OFDError(RuntimeError):
    """A libofd call returned an error status."""


class ofd_config(ctypes.Structure):
    _fields_ = [('dim', ctypes.c_int * 3),
                ('space_order', ctypes.c_int),
                ('storage', ctypes.c_int),
                ('legacy_bc', ctypes.c_int),
                ('free_surface', ctypes.c_int * 6),
                ('spacing', ctypes.c_double * 3),
                ('dt', ctypes.c_double),
                ('weights', ctypes.c_double * 4),
                ('field_scale', ctypes.c_float * 9),
                ('kernel_variant', ctypes.c_int),
                ('rounding', ctypes.c_int)]


REGULAR_MAX_TERMS = 96


class ofd_regular_config(ctypes.Structure):
    _fields_ = [('dim', ctypes.c_int * 3),
                ('margin', ctypes.c_int),
                ('storage', ctypes.c_int),
                ('nterms', ctypes.c_int),
                ('level', ctypes.c_int * REGULAR_MAX_TERMS),
                ('offset', (ctypes.c_int * 3) * REGULAR_MAX_TERMS),
                ('coef', ctypes.c_double * REGULAR_MAX_TERMS),
                ('variant', ctypes.c_int)]


class ofd_field_view(ctypes.Structure):
    _fields_ = [('base', ctypes.c_void_p), ('pitch', ctypes.c_long),
                ('storage', ctypes.c_int), ('scale', ctypes.c_float)]


_lib = None


def library_path():
    return _build.LIBNAME


def load_library():
    """Load lib/libofd.so.  The library is built by ``__graft_entry__.build()``
    (or ``python opesci-fd_gb300/opesci/build.py``); a missing library is an
    error, never a fallback."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIBNAME
    if not os.path.exists(path):
        raise OFDError('libofd.so not built (%s); run __graft_entry__.build()' % path)
    lib = ctypes.CDLL(path, mode=ctypes.RTLD_GLOBAL)
    P = ctypes.POINTER
    h = ctypes.c_void_p
    fptr = P(ctypes.c_float)
    sig = {
        'ofd_create': [P(ofd_config), P(h)],
        'ofd_destroy': [h],
        'ofd_footprint': [P(ofd_config), P(ctypes.c_size_t)],
        'ofd_set_media_const': [h, ctypes.c_float, ctypes.c_float, ctypes.c_float],
        'ofd_set_coefficients': [h, ctypes.c_int, fptr, ctypes.c_int, fptr, ctypes.c_int],
        'ofd_set_ghost_coefficients': [h, ctypes.c_int, fptr, ctypes.c_int],
        'ofd_set_media': [h, fptr, fptr, fptr],
        'ofd_set_media_async': [h, fptr, fptr, fptr],
        'ofd_upload_field': [h, ctypes.c_int, ctypes.c_int, fptr],
        'ofd_download_field': [h, ctypes.c_int, ctypes.c_int, fptr],
        'ofd_upload_field_f64': [h, ctypes.c_int, ctypes.c_int, P(ctypes.c_double)],
        'ofd_download_field_f64': [h, ctypes.c_int, ctypes.c_int, P(ctypes.c_double)],
        'ofd_upload_field_async': [h, ctypes.c_int, ctypes.c_int, fptr],
        'ofd_download_field_async': [h, ctypes.c_int, ctypes.c_int, fptr],
        'ofd_upload_field_device': [h, ctypes.c_int, ctypes.c_int, ctypes.c_void_p],
        'ofd_download_field_device': [h, ctypes.c_int, ctypes.c_int, ctypes.c_void_p],
        'ofd_zero_fields': [h],
        'ofd_set_source': [h, ctypes.c_int, ctypes.c_int, ctypes.c_int, fptr, ctypes.c_int],
        'ofd_set_source_xyz': [h, ctypes.c_int, ctypes.c_int, ctypes.c_int, fptr, fptr, fptr, ctypes.c_int],
        'ofd_set_receivers': [h, ctypes.c_int, P(ctypes.c_int), ctypes.c_int],
        'ofd_get_traces': [h, fptr],
        'ofd_apply_boundary_init': [h, ctypes.c_int],
        'ofd_step': [h, ctypes.c_int],
        'ofd_step_graph': [h, ctypes.c_int],
        'ofd_set_persistent': [h, ctypes.c_int],
        'ofd_set_wait_limit': [h, ctypes.c_double],
        'ofd_set_ghost_schedule': [h, ctypes.c_int, ctypes.c_int],
        'ofd_step_timed': [h, ctypes.c_int, P(ctypes.c_double), P(ctypes.c_long)],
        'ofd_set_tuning': [h, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int],
        'ofd_step_profiled': [h, ctypes.c_int, P(ctypes.c_double), P(ctypes.c_double), P(ctypes.c_long)],
        'ofd_sync': [h],
        'ofd_query': [h],
        'ofd_get_step': [h, P(ctypes.c_long)],
        'ofd_set_step': [h, ctypes.c_long],
        'ofd_field_sumsq': [h, ctypes.c_int, P(ctypes.c_double)],
        'ofd_field_absmax': [h, ctypes.c_int, P(ctypes.c_double)],
        'ofd_field_view_get': [h, ctypes.c_int, ctypes.c_int, P(ofd_field_view)],
        'ofd_group_create': [P(h), ctypes.c_int, ctypes.c_int, P(h)],
        'ofd_group_step': [h, ctypes.c_int],
        'ofd_set_device': [ctypes.c_int],
        'ofd_group_eligible': [h],
        'ofd_segy_decode_ibm': [ctypes.c_void_p, ctypes.c_long, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                ctypes.c_int, fptr],
        'ofd_write_field_vts_3d': [ctypes.c_char_p, P(ctypes.c_int), fptr, ctypes.c_int, fptr],
        'ofd_group_query': [h],
        'ofd_group_sync': [h],
        'ofd_group_destroy': [h],
        'ofd_regular_create': [P(ofd_regular_config), P(h)],
        'ofd_regular_destroy': [h],
        'ofd_regular_upload': [h, ctypes.c_int, ctypes.c_void_p],
        'ofd_regular_download': [h, ctypes.c_int, ctypes.c_void_p],
        'ofd_regular_upload_device': [h, ctypes.c_int, ctypes.c_void_p],
        'ofd_regular_download_device': [h, ctypes.c_int, ctypes.c_void_p],
        'ofd_regular_step': [h, ctypes.c_int],
        'ofd_regular_step_timed': [h, ctypes.c_int, P(ctypes.c_double)],
        'ofd_regular_get_step': [h, P(ctypes.c_long)],
        'ofd_regular_set_step': [h, ctypes.c_long],
        'ofd_regular_sync': [h],
    }
    for name, args in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = ctypes.c_int
    lib.ofd_last_error.argtypes = []
    lib.ofd_last_error.restype = ctypes.c_char_p
    lib.ofd_stream.argtypes = [h]
    lib.ofd_stream.restype = ctypes.c_void_p
    lib.ofd_regular_stream.argtypes = [h]
    lib.ofd_regular_stream.restype = ctypes.c_void_p
    lib.ofd_sumsq_field_noalloc.argtypes = [ctypes.c_void_p, P(ctypes.c_int), ctypes.c_int, ctypes.c_void_p,
                                            ctypes.c_void_p]
    lib.ofd_sumsq_field_noalloc.restype = ctypes.c_int
    lib.ofd_noalloc_last_error.argtypes = []
    lib.ofd_noalloc_last_error.restype = ctypes.c_char_p
    _lib = lib
    return lib


def set_device(index):
    """Device of the simulations this thread creates next (one process per
    GPU passes its local rank)."""
    lib = load_library()
    _check(lib.ofd_set_device(int(index)), 'ofd_set_device')


def _check(rc, what):
    if rc != 0:
        msg = _lib.ofd_last_error().decode(errors='replace')
        raise OFDError('%s failed (%d): %s' % (what, rc, msg))


def _fptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


ROUNDING = {'nearest': 0, 'stochastic': 1}


def make_config(dims, space_order, spacing, dt, weights, storage='f32', free_surface=None,
                legacy_bc=False, field_scale=None, kernel_variant=0, rounding='nearest'):
    cfg = ofd_config()
    for i in range(3):
        cfg.dim[i] = int(dims[i])
        cfg.spacing[i] = float(spacing[i])
    cfg.space_order = int(space_order)
    cfg.storage = STORAGE[storage] if isinstance(storage, str) else int(storage)
    cfg.legacy_bc = 1 if legacy_bc else 0
    fs = free_surface if free_surface is not None else [0] * 6
    for i in range(6):
        v = fs[i]
        cfg.free_surface[i] = BC[v] if isinstance(v, str) else int(v)
    cfg.dt = float(dt)
    for k in range(4):
        cfg.weights[k] = float(weights[k]) if k < len(weights) else 0.0
    for f in range(9):
        cfg.field_scale[f] = float(field_scale[f]) if field_scale is not None else 1.0
    cfg.kernel_variant = int(kernel_variant)
    cfg.rounding = ROUNDING[rounding] if isinstance(rounding, str) else int(rounding)
    return cfg


def config_from_grid(grid, storage=None, kernel_variant=0, field_scale=None, rounding='nearest'):
    """ofd_config of a solved StaggeredGrid: dims, margin, spacing, dt, the
    staggered weights of its space order, per-face free-surface algorithms."""
    faces = [0] * 6
    fs = getattr(grid, 'free_surface', {})
    for (dim, side), algo in fs.items():
        faces[2 * (dim - 1) + side] = BC[algo]
    if storage is None:
        storage = 'f64' if grid.double else 'f32'
    return make_config([d.value for d in grid.dim], grid.order[1], [s.value for s in grid.spacing],
                       grid.dt.value, grid.fd_weights(), storage=storage, free_surface=faces,
                       legacy_bc=getattr(grid, 'legacy_bc', False), field_scale=field_scale,
                       kernel_variant=kernel_variant, rounding=rounding)


class Simulation(object):
    """One device-resident elastic simulation (a libofd handle)."""

    def __init__(self, cfg):
        self.lib = load_library()
        self.cfg = cfg
        self.dims = tuple(cfg.dim[i] for i in range(3))
        self.h = ctypes.c_void_p()
        _check(self.lib.ofd_create(ctypes.byref(cfg), ctypes.byref(self.h)), 'ofd_create')

    @staticmethod
    def footprint(cfg):
        lib = load_library()
        n = ctypes.c_size_t()
        _check(lib.ofd_footprint(ctypes.byref(cfg), ctypes.byref(n)), 'ofd_footprint')
        return n.value

    def close(self):
        if self.h:
            self.lib.ofd_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _arr(self, a):
        a = np.ascontiguousarray(a, dtype=np.float32)
        if a.shape != self.dims:
            a = a.reshape(self.dims)
        return a

    def set_coefficients(self, het, ks, kv):
        ks = np.ascontiguousarray(ks, dtype=np.float32)
        kv = np.ascontiguousarray(kv, dtype=np.float32)
        _check(self.lib.ofd_set_coefficients(self.h, int(het), _fptr(ks), len(ks), _fptr(kv), len(kv)),
               'ofd_set_coefficients')

    def set_coefficients_from_grid(self, grid):
        """Literal tables of the grid's generated update expressions, after
        checking that their structure is the prebuilt one."""
        from .templates import cuda_gen
        # with the expand or eval_const switch off, the same update in the
        # default printed form (cuda_gen.default_form)
        tabs, _ = cuda_gen.model_tables(grid)
        key = 'so%d_%s' % (grid.order[1], 'het' if grid.read else 'const')
        pre = cuda_gen.prebuilt_signatures().get(key)
        if pre is None or pre['stress'] != tabs['stress'][0] or pre['velocity'] != tabs['velocity'][0]:
            raise OFDError('the update expressions of this model (%s) do not match the prebuilt '
                           'CUDA expressions; regenerate csrc/generated' % key)
        self.set_coefficients(1 if grid.read else 0, tabs['stress'][1], tabs['velocity'][1])
        self.set_ghost_coefficients_from_grid(grid)

    def set_ghost_coefficients(self, het, kg):
        kg = np.ascontiguousarray(kg, dtype=np.float32)
        _check(self.lib.ofd_set_ghost_coefficients(self.h, int(het), _fptr(kg), len(kg)),
               'ofd_set_ghost_coefficients')

    def set_het_ghost_coefficients(self):
        """For a heterogeneous (read-mode) model of space order 4 with
        Levander faces and isotropic spacing, the ghost literal table from
        the stored monomials (cuda_gen.het_ghost_table) without the symbolic
        frontend; other models keep the restated ghost formulas.  Returns
        True when set."""
        from .templates import cuda_gen
        c = self.cfg
        if (c.space_order != 4 or c.storage == STORAGE['f64']
                or any(c.free_surface[i] != BC['levander'] for i in range(6))
                or not (c.spacing[0] == c.spacing[1] == c.spacing[2])):
            return False
        self.set_ghost_coefficients(1, cuda_gen.het_ghost_table(c.dt, c.spacing[0]))
        return True

    def set_ghost_coefficients_from_grid(self, grid):
        """Space order 4 with Levander faces: evaluate the ghosts from the
        grid's own printed ghost equations when their structure is the
        prebuilt one (FP32/FP16/BF16 storage).  Returns True when set."""
        from .templates import cuda_gen
        if self.cfg.storage == STORAGE['f64']:
            return False
        tab = cuda_gen.model_ghost_table(grid)
        if tab is None:
            return False
        key = 'so4_%s' % ('het' if grid.read else 'const')
        pre = cuda_gen.prebuilt_signatures().get(key, {})
        if pre.get('ghost') != tab[0]:
            return False
        self.set_ghost_coefficients(1 if grid.read else 0, tab[1])
        return True

    def set_media_const(self, beta, lam, mu):
        _check(self.lib.ofd_set_media_const(self.h, beta, lam, mu), 'ofd_set_media_const')

    def set_media(self, rho, vp, vs):
        r, p, s = self._arr(rho), self._arr(vp), self._arr(vs)
        _check(self.lib.ofd_set_media(self.h, _fptr(r), _fptr(p), _fptr(s)), 'ofd_set_media')

    @property
    def host_dtype(self):
        """Element type of upload()/download() arrays: float64 for FP64
        storage, else float32."""
        return np.float64 if self.cfg.storage == STORAGE['f64'] else np.float32

    def upload(self, field, level, array):
        f = FIELDS.index(field) if isinstance(field, str) else field
        if self.host_dtype == np.float64:
            a = np.ascontiguousarray(array, dtype=np.float64).reshape(self.dims)
            _check(self.lib.ofd_upload_field_f64(self.h, f, level, a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))),
                   'ofd_upload_field_f64')
            return
        a = self._arr(array)
        _check(self.lib.ofd_upload_field(self.h, f, level, _fptr(a)), 'ofd_upload_field')

    def download(self, field, level=None):
        """One field level in the reference layout: float64 for FP64 storage
        (exact), else float32."""
        f = FIELDS.index(field) if isinstance(field, str) else field
        if level is None:
            level = self.steps % 2
        out = np.empty(self.dims, dtype=self.host_dtype)
        if out.dtype == np.float64:
            _check(self.lib.ofd_download_field_f64(self.h, f, level, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))),
                   'ofd_download_field_f64')
        else:
            _check(self.lib.ofd_download_field(self.h, f, level, _fptr(out)), 'ofd_download_field')
        return out

    def download_all_async(self, outs, level=None):
        """Queue the download of all nine fields of a level into ``outs``
        (nine float32 arrays of the grid's dims, ideally pinned); they are
        filled once sync() returns."""
        if level is None:
            level = self.steps % 2
        for i, o in enumerate(outs):
            if o.dtype != np.float32 or o.shape != self.dims or not o.flags['C_CONTIGUOUS']:
                raise ValueError('download buffers must be C-contiguous float32 arrays of shape %s' % (self.dims,))
            _check(self.lib.ofd_download_field_async(self.h, i, level, _fptr(o)), 'ofd_download_field_async')

    def set_media_async(self, rho, vp, vs):
        """ofd_set_media queued without waiting; the arrays must stay alive
        (and unchanged) until sync()."""
        arrs = [np.asarray(a) for a in (rho, vp, vs)]
        for a in arrs:
            if a.dtype != np.float32 or a.shape != self.dims or not a.flags['C_CONTIGUOUS']:
                raise ValueError('media arrays must be C-contiguous float32 arrays of shape %s' % (self.dims,))
        _check(self.lib.ofd_set_media_async(self.h, *[_fptr(a) for a in arrs]), 'ofd_set_media_async')

    def zero(self):
        _check(self.lib.ofd_zero_fields(self.h), 'ofd_zero_fields')

    def set_source(self, pos, wavelet):
        """Point source at array index ``pos``: one signal for all three normal
        stresses, or a triple (x, y, z) of equally long signals."""
        w = np.asarray(wavelet, dtype=np.float32)
        if w.ndim == 2:
            if w.shape[0] != 3:
                raise ValueError('three source signals (x, y, z) expected, got shape %s' % (w.shape,))
            sx, sy, sz = (np.ascontiguousarray(w[q]) for q in range(3))
            _check(self.lib.ofd_set_source_xyz(self.h, int(pos[0]), int(pos[1]), int(pos[2]), _fptr(sx),
                                               _fptr(sy), _fptr(sz), w.shape[1]), 'ofd_set_source_xyz')
            return
        w = np.ascontiguousarray(w.reshape(-1))
        _check(self.lib.ofd_set_source(self.h, int(pos[0]), int(pos[1]), int(pos[2]), _fptr(w), len(w)),
               'ofd_set_source')

    def set_receivers(self, ijk, nt_cap):
        """Record U, V, W and P = (Txx+Tyy+Tzz)/3 at array indices ``ijk``
        ((n, 3), margins included) after every step, for up to nt_cap steps."""
        a = np.ascontiguousarray(np.asarray(ijk, dtype=np.int32).reshape(-1, 3))
        self._nrec, self._rec_cap = len(a), int(nt_cap)
        _check(self.lib.ofd_set_receivers(self.h, len(a), a.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                          int(nt_cap)), 'ofd_set_receivers')

    def traces(self):
        """Recorded traces, shape (nt_cap, 4, nrec): U, V, W, P per step."""
        out = np.empty((self._rec_cap, 4, self._nrec), dtype=np.float32)
        _check(self.lib.ofd_get_traces(self.h, _fptr(out)), 'ofd_get_traces')
        return out

    def boundary_init(self, level=0):
        _check(self.lib.ofd_apply_boundary_init(self.h, level), 'ofd_apply_boundary_init')

    def step(self, n=1):
        _check(self.lib.ofd_step(self.h, int(n)), 'ofd_step')

    def step_graph(self, n):
        """Advance n steps by replaying a captured two-step CUDA graph."""
        _check(self.lib.ofd_step_graph(self.h, int(n)), 'ofd_step_graph')

    def step_timed(self, n):
        """n steps on the launch path, timed with CUDA events on the
        handle's stream only around all of them: (ms, kernel launches)."""
        ms = ctypes.c_double()
        nl = ctypes.c_long()
        _check(self.lib.ofd_step_timed(self.h, int(n), ctypes.byref(ms), ctypes.byref(nl)), 'ofd_step_timed')
        return ms.value, nl.value

    def set_persistent(self, enable=True):
        """Run time steps in cooperative launches of up to 1024 steps."""
        _check(self.lib.ofd_set_persistent(self.h, 1 if enable else 0), 'ofd_set_persistent')

    def set_wait_limit(self, seconds):
        """Limit of every device-side wait of this simulation's kernels (TMA
        pipeline waits, grid barriers); expiry makes the next sync raise
        OFDError with code OFD_ETIMEOUT."""
        _check(self.lib.ofd_set_wait_limit(self.h, float(seconds)), 'ofd_set_wait_limit')

    def set_ghost_schedule(self, mode, blocks_per_sm):
        """Where the generated space-order-4 ghosts' recompute runs: mode 0
        after the stress sweep, 1 beside it on a high-priority stream;
        blocks_per_sm sizes its grid.  Results do not depend on either."""
        _check(self.lib.ofd_set_ghost_schedule(self.h, int(mode), int(blocks_per_sm)), 'ofd_set_ghost_schedule')

    def set_tuning(self, stress_variant=0, velocity_variant=0, chunk_waves=1, plain_bx=32, plain_by=8,
                   persistent=0, rc_mode=None, rc_bps=None):
        """Apply autotuner knobs (opesci.autotune); rc_mode / rc_bps, when
        given, set the generated ghosts' recompute schedule."""
        _check(self.lib.ofd_set_tuning(self.h, int(stress_variant), int(velocity_variant), int(chunk_waves),
                                       int(plain_bx), int(plain_by)), 'ofd_set_tuning')
        self.set_persistent(bool(persistent))
        if rc_mode is not None:
            self.set_ghost_schedule(rc_mode, 4 if rc_bps is None else rc_bps)

    def step_profiled(self, n):
        """Advance n steps with CUDA events on the handle's stream; returns
        (total ms, [stress sweep, stress ghosts, velocity sweep, velocity
        ghosts] ms, kernel launches)."""
        tot = ctypes.c_double()
        cls = (ctypes.c_double * 4)()
        nl = ctypes.c_long()
        _check(self.lib.ofd_step_profiled(self.h, int(n), ctypes.byref(tot), cls, ctypes.byref(nl)),
               'ofd_step_profiled')
        return tot.value, list(cls), nl.value

    def done(self):
        """True when all work queued on this simulation has finished."""
        rc = self.lib.ofd_query(self.h)
        if rc < 0:
            _check(rc, 'ofd_query')
        return rc == 0

    def sync(self):
        _check(self.lib.ofd_sync(self.h), 'ofd_sync')

    def groupable(self):
        """True when this simulation may join a Group (tiled sweeps apply)."""
        rc = self.lib.ofd_group_eligible(self.h)
        if rc < 0:
            _check(rc, 'ofd_group_eligible')
        return rc == 1

    @property
    def steps(self):
        v = ctypes.c_long()
        _check(self.lib.ofd_get_step(self.h, ctypes.byref(v)), 'ofd_get_step')
        return v.value

    @steps.setter
    def steps(self, n):
        _check(self.lib.ofd_set_step(self.h, int(n)), 'ofd_set_step')

    def sumsq(self, level=None):
        if level is None:
            level = self.steps % 2
        out = (ctypes.c_double * 9)()
        _check(self.lib.ofd_field_sumsq(self.h, level, out), 'ofd_field_sumsq')
        return np.array(list(out))

    def absmax(self, level=None):
        if level is None:
            level = self.steps % 2
        out = (ctypes.c_double * 9)()
        _check(self.lib.ofd_field_absmax(self.h, level, out), 'ofd_field_absmax')
        return np.array(list(out))

    @property
    def stream(self):
        return self.lib.ofd_stream(self.h)

    def view(self, field, level):
        v = ofd_field_view()
        f = FIELDS.index(field) if isinstance(field, str) else field
        _check(self.lib.ofd_field_view_get(self.h, f, level, ctypes.byref(v)), 'ofd_field_view_get')
        return v


class Solo(object):
    """A simulation stepped on its own stream, with the Group interface
    (done/sync/close) so that drivers can mix it with groups."""

    def __init__(self, sim):
        self.sims = [sim]

    def step(self, n):
        self.sims[0].step_graph(n)

    def done(self):
        return self.sims[0].done()

    def sync(self):
        self.sims[0].sync()

    def close(self):
        pass


def make_groups(sims, chunk_planes=0):
    """Group and Solo objects covering ``sims`` (which share space order,
    storage, media mode and time level): one Group of every simulation that
    may join one, a Solo for each other."""
    ok = [s for s in sims if s.groupable()]
    out = [Group(ok, chunk_planes=chunk_planes)] if ok else []
    return out + [Solo(s) for s in sims if not s.groupable()]


class Group(object):
    """Simulations advanced together (ofd_group): every phase of a step is
    one launch over all members, replayed from a captured two-step graph.
    Members must share space order, storage and media mode and stand at the
    same time level; create the group after configuring them (media,
    coefficients, source), and close it before closing a member."""

    def __init__(self, sims, chunk_planes=0):
        self.lib = load_library()
        self.sims = list(sims)
        arr = (ctypes.c_void_p * len(self.sims))(*[s.h.value for s in self.sims])
        self.g = ctypes.c_void_p()
        _check(self.lib.ofd_group_create(arr, len(self.sims), int(chunk_planes), ctypes.byref(self.g)),
               'ofd_group_create')

    def step(self, n):
        _check(self.lib.ofd_group_step(self.g, int(n)), 'ofd_group_step')

    def done(self):
        rc = self.lib.ofd_group_query(self.g)
        if rc < 0:
            _check(rc, 'ofd_group_query')
        return rc == 0

    def sync(self):
        _check(self.lib.ofd_group_sync(self.g), 'ofd_group_sync')

    def close(self):
        if self.g:
            self.lib.ofd_group_destroy(self.g)
            self.g = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


# --------------------------------------------------------------- regular grid

def regular_config(dims, margin, terms, storage='f32', variant=0):
    """ofd_regular_config from padded dims, the margin and a term table
    [(level, (dx, dy, dz), coef), ...] (level 1: t, 0: t-1); variant 0 is
    the direct sweep, 1 the shared-memory ring sweep."""
    st = {'f32': 0, 'float': 0, 'fp32': 0, 'f64': 3, 'double': 3, 'fp64': 3}.get(storage)
    if st is None:
        raise ValueError('regular-grid storage must be f32 or f64, not %r' % storage)
    if not 1 <= len(terms) <= REGULAR_MAX_TERMS:
        raise ValueError('%d terms (1..%d supported)' % (len(terms), REGULAR_MAX_TERMS))
    cfg = ofd_regular_config()
    for i in range(3):
        cfg.dim[i] = int(dims[i])
    cfg.margin = int(margin)
    cfg.storage = st
    cfg.nterms = len(terms)
    for k, (lvl, off, coef) in enumerate(terms):
        cfg.level[k] = int(lvl)
        for d in range(3):
            cfg.offset[k][d] = int(off[d])
        cfg.coef[k] = float(coef)
    cfg.variant = int(variant)
    return cfg


def regular_config_from_grid(grid, variant=0):
    """The device configuration of a solved one-field RegularGrid."""
    from .templates.regular_tmpl import model_terms
    if len(grid.fields) != 1:
        raise ValueError('the regular-grid device runtime advances one field')
    terms = model_terms(grid, grid.fields[0])
    return regular_config([d.value for d in grid.dim], grid.margin.value, terms,
                          'f64' if grid.double else 'f32', variant=variant)


class RegularSimulation(object):
    """One regular-grid (acoustic) field on three time levels resident in HBM
    (ofd_regular_*).  Level arrays are real_t[dim1][dim2][dim3]; step n
    writes level (n % 3 + 2) % 3 from levels n % 3 (t-1) and (n % 3 + 1) % 3
    (t), like the reference's _t0/_t1/_t2 rotation."""

    def __init__(self, cfg):
        self.lib = load_library()
        self.cfg = cfg
        self.dims = tuple(cfg.dim)
        self.dtype = np.float64 if cfg.storage == 3 else np.float32
        self.h = ctypes.c_void_p()
        _check(self.lib.ofd_regular_create(ctypes.byref(cfg), ctypes.byref(self.h)), 'ofd_regular_create')

    def upload(self, level, arr):
        a = np.ascontiguousarray(arr, dtype=self.dtype)
        if a.shape != self.dims:
            raise ValueError('level shape %s, expected %s' % (a.shape, self.dims))
        _check(self.lib.ofd_regular_upload(self.h, int(level), a.ctypes.data), 'ofd_regular_upload')

    def download(self, level):
        a = np.empty(self.dims, dtype=self.dtype)
        _check(self.lib.ofd_regular_download(self.h, int(level), a.ctypes.data), 'ofd_regular_download')
        return a

    def step(self, n):
        _check(self.lib.ofd_regular_step(self.h, int(n)), 'ofd_regular_step')

    def step_timed(self, n):
        """Milliseconds of n steps measured by CUDA events on the handle's stream."""
        ms = ctypes.c_double()
        _check(self.lib.ofd_regular_step_timed(self.h, int(n), ctypes.byref(ms)), 'ofd_regular_step_timed')
        return ms.value

    @property
    def steps(self):
        v = ctypes.c_long()
        _check(self.lib.ofd_regular_get_step(self.h, ctypes.byref(v)), 'ofd_regular_get_step')
        return v.value

    @steps.setter
    def steps(self, n):
        _check(self.lib.ofd_regular_set_step(self.h, int(n)), 'ofd_regular_set_step')

    def newest_level(self):
        """Level written by the last step (level 1 before any step)."""
        n = self.steps
        return 1 if n == 0 else ((n - 1) % 3 + 2) % 3

    def sync(self):
        _check(self.lib.ofd_regular_sync(self.h), 'ofd_regular_sync')

    def close(self):
        if self.h:
            self.lib.ofd_regular_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
