"""Compilers for generated programs (restates opesci/compilation.py:10-104
with a CUDA target).

NVCCCompiler builds the CUDA program emitted by the grid's template into a
shared library (or an executable) for sm_103a, linked against the device
runtime libofd.so.  This backend has no CPU target: the GNU/Clang/Intel
compiler names of the reference select a CPU OpenMP build, which this package
does not provide, and are rejected with an error."""
import os
import shutil
import subprocess

from . import build as _build

__all__ = ['Compiler', 'NVCCCompiler', 'get_package_dir', 'compiler_for']


def get_package_dir():
    return os.path.abspath(os.path.dirname(__file__))


class Compiler(object):
    """Runs a compiler subprocess into a shared library or executable and
    writes a log next to the source (compilation.py:26-48)."""

    def __init__(self, cc, cppargs=(), ldargs=()):
        self._cc = os.environ.get('NVCC', cc)
        self._cppargs = list(cppargs)
        self._ldargs = list(ldargs)

    # language flag placed before the source (nvcc: '-x cu', so that a
    # program written to a .cpp file, as the reference's model scripts name
    # it, still compiles as CUDA)
    _src_lang = ()

    def compile(self, src, out=None, shared=True):
        basename = os.path.splitext(src)[0]
        outname = out or ('%s.so' % basename if shared else basename)
        cpp = list(self._cppargs) + (['-Xcompiler', '-fPIC'] if shared else [])
        ld = (['-shared'] if shared else []) + list(self._ldargs)
        cmd = [self._cc] + cpp + ['-o', outname] + list(self._src_lang) + [src] + ld
        with open('%s.log' % basename, 'w') as log:
            log.write('Compiling: %s\n' % ' '.join(cmd))
            log.flush()
            try:
                subprocess.check_call(cmd, stdout=log, stderr=log)
            except OSError:
                raise RuntimeError('OSError during compilation\nPlease check if compiler exists: %s' % self._cc)
            except subprocess.CalledProcessError:
                raise RuntimeError('Error during compilation:\nCompilation command: %s\nSource file: %s\n'
                                   'Log file: %s' % (' '.join(cmd), src, log.name))
        return outname


class NVCCCompiler(Compiler):
    """nvcc for sm_103a, linked against lib/libofd.so with an rpath."""

    _src_lang = ('-x', 'cu')

    def __init__(self, cppargs=(), ldargs=()):
        lib = _build.build()   # the device runtime must exist before linking
        libdir = os.path.dirname(lib)
        exe = shutil.which('nvcc') or '/usr/local/cuda/bin/nvcc'
        opt = ['-gencode', 'arch=compute_103a,code=sm_103a', '-O3', '-std=c++17', '-fmad=false',
               '-I%s' % _build.INCLUDE]
        link = ['-L%s' % libdir, '-lofd', '-Xlinker', '-rpath=%s' % libdir]
        super().__init__(exe, cppargs=opt + list(cppargs), ldargs=link + list(ldargs))


def compiler_for(name):
    if name in ('nvcc', 'cuda', 'nvidia', None):
        return NVCCCompiler()
    if name in ('g++', 'gnu', 'clang', 'clang++', 'icpc', 'intel'):
        raise ValueError('compiler %r selects the CPU OpenMP target, which this GB300 backend does not '
                         'provide; use compiler="nvcc"' % name)
    raise ValueError('Unknown compiler.')
