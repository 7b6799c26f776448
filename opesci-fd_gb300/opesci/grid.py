"""Grid base: generate, compile, execute, convergence (restates
opesci/grid.py:8-156 on the CUDA target).

The generated program exports the reference's C ABI: opesci_execute(grid,
profiling), opesci_convergence(grid, conv) and opesci_free(grid) over the
OpesciGrid / OpesciConvergence / OpesciProfiling structs, so execution goes
through ctypes exactly as in the reference."""
import ctypes
import os
from ctypes import Structure, POINTER, c_float, c_double, pointer

from .codeprinter import ccode

__all__ = ['Grid']


class Grid(object):
    """Code generation, compilation and execution of a grid's program."""

    src_code = None
    src_file = None
    src_lib = None
    _library = None
    _arg_grid = None
    _arg_conv = None
    _compiler_name = 'nvcc'

    def __init__(self):
        pass

    def _load_library(self, src_lib=None):
        libname = src_lib or self.src_lib
        try:
            self._library = ctypes.cdll.LoadLibrary(os.path.abspath(libname))
        except OSError as e:
            raise Exception('Failed to load %s: %s' % (libname, e))

    @property
    def compiler(self):
        from .compilation import compiler_for
        return compiler_for(self._compiler_name)

    @compiler.setter
    def compiler(self, compiler):
        from .compilation import compiler_for
        compiler_for(compiler)          # validates; raises for CPU targets
        self._compiler_name = compiler

    def generate(self, filename, compiler=None):
        """Write the generated CUDA program to ``filename``."""
        if compiler:
            self.compiler = compiler
        self.src_code = self.cgen_template.generate()
        self.src_file = filename
        with open(self.src_file, 'w') as f:
            f.write(self.src_code)
        print('Generated:', self.src_file)

    def compile(self, filename, compiler=None, shared=True):
        """Generate (if needed) and build the program with nvcc."""
        if compiler:
            self.compiler = compiler
        if self.src_file is None or self.src_file != filename:
            self.generate(filename)
        out = self.compiler.compile(self.src_file, shared=shared)
        if shared:
            self.src_lib = out
        print('Compiled:', out)
        return out

    def pluto_op(self, filename):
        """The reference runs polycc over the generated C for tiled OpenMP
        loops (grid.py:158-180).  Loop tiling of the CUDA program belongs to
        the device runtime (TMA tiles, chunking chosen by opesci.autotune),
        so the program is returned unchanged."""
        print('Pluto tiling does not apply to the CUDA target; using %s as generated' % filename)
        return filename

    def _real(self):
        return c_double if getattr(self, 'double', False) else c_float

    def execute(self, filename, compiler='nvcc', nthreads=1, affinity='close'):
        """Compile if needed, load, and run opesci_execute (grid.py:85-130).
        ``nthreads``/``affinity`` are accepted for compatibility; the time loop
        runs on the GPU."""
        if self.src_lib is None:
            self.compile(filename, compiler=compiler, shared=True)
        self._load_library(src_lib=self.src_lib)
        real = self._real()

        class OpesciGrid(Structure):
            _fields_ = [(ccode(f.label), POINTER(real)) for f in self.fields]

        class OpesciProfiling(Structure):
            _fields_ = [(v, c_float) for v in ('rtime', 'ptime', 'mflops')]
            _fields_ += [(ev, ctypes.c_longlong) for ev in getattr(self, '_papi_events', [])]

        self._arg_grid = OpesciGrid()
        self._arg_profiling = OpesciProfiling()
        fn = self._library.opesci_execute
        fn.argtypes = [POINTER(OpesciGrid), POINTER(OpesciProfiling)]
        fn.restype = ctypes.c_int
        print('Executing on the GPU')
        rc = fn(pointer(self._arg_grid), pointer(self._arg_profiling))
        if rc != 0:
            raise RuntimeError('opesci_execute failed with status %d' % rc)
        if self.profiling:
            # the reference's report (grid.py:122-130); the time is the GPU time
            # loop's (CUDA events) and MFlops/s counts the update expressions'
            # operations, PAPI counters being host-CPU events
            for ev in getattr(self, '_papi_events', []):
                print('PAPI:: %s: not counted on the GPU' % ev)
            print('GPU time loop: %f (sec)' % self._arg_profiling.rtime)
            print('Max real_time: %f (sec)' % self._arg_profiling.rtime)
            print('Max proc_time: %f (sec)' % self._arg_profiling.ptime)
            print('Total MFlops/s: %f' % self._arg_profiling.mflops)

    def convergence(self):
        """L2 norms against the analytic solution (grid.py:132-156)."""
        if self._library is None:
            self._load_library()
        if self._arg_grid is None:
            raise RuntimeError('Convergence could not find grid argument!\nYou need to you run grid.execute() first!')
        real = self._real()

        class OpesciConvergence(Structure):
            _fields_ = [('%s_l2' % ccode(f.label), real) for f in self.fields]

        arg = OpesciConvergence()
        fn = self._library.opesci_convergence
        fn.argtypes = [POINTER(self._arg_grid.__class__), POINTER(OpesciConvergence)]
        fn.restype = ctypes.c_int
        print('Convergence:')
        rc = fn(pointer(self._arg_grid), pointer(arg))
        if rc != 0:
            raise RuntimeError('opesci_convergence failed with status %d' % rc)
        out = {}
        for name, _ in arg._fields_:
            out[name] = getattr(arg, name)
            print('%s: %.10f' % (name, out[name]))
        self.l2 = out
        return out

    def field_array(self, name, level=None):
        """The published host array of a field after execute(), as NumPy
        (reference layout [levels][dim1][dim2][dim3]: two levels for the
        elastic scheme, three for the regular one); ``level`` selects one."""
        import numpy as np
        if self._arg_grid is None:
            raise RuntimeError('run execute() first')
        dims = [d.value for d in self.dim]
        ptr = getattr(self._arg_grid, name)
        dtype = np.float64 if getattr(self, 'double', False) else np.float32
        arr = np.ctypeslib.as_array(ptr, shape=(len(self.time),) + tuple(dims)).astype(dtype, copy=True)
        return arr if level is None else arr[level]

    def free(self):
        if self._library is not None and self._arg_grid is not None:
            fn = self._library.opesci_free
            fn.argtypes = [POINTER(self._arg_grid.__class__)]
            fn(pointer(self._arg_grid))
            self._arg_grid = None
