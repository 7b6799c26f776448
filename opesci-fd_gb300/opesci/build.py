"""Build the device runtime libofd.so in-tree with nvcc for sm_103a.

Each translation unit of csrc/ is compiled in parallel; objects and the
library land in opesci-fd_gb300/lib/ (git-ignored)."""
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REPO_ROOT = os.path.dirname(PKG_ROOT)
CSRC = os.path.join(PKG_ROOT, 'csrc')
LIBDIR = os.path.join(PKG_ROOT, 'lib')
INCLUDE = os.path.join(REPO_ROOT, 'include')
LIBNAME = os.path.join(LIBDIR, 'libofd.so')

ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
# -fmad=false: no multiply-add contraction, so the generated update
# expressions round exactly like the reference's C code (which g++ does not
# contract in ISO C++ mode)
NVCC_FLAGS = ['-O3', '-lineinfo', '-std=c++17', '-Xcompiler', '-fPIC', '--expt-relaxed-constexpr',
              '-fmad=false', '-Xptxas', '-warn-spills']


def nvcc():
    exe = shutil.which('nvcc')
    if exe is None and os.path.exists('/usr/local/cuda/bin/nvcc'):
        exe = '/usr/local/cuda/bin/nvcc'
    if exe is None:
        raise RuntimeError('nvcc not found: the CUDA toolkit is required to build libofd')
    return exe


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith('.cu'))


def jobs():
    """(source, object, extra flags) per translation unit: ofd_inst_*.cu (the
    kernels of one storage type) once per radius 1..4, the rest once."""
    out = []
    for src in sources():
        base = os.path.basename(src)[:-3]
        if base.startswith('ofd_inst_'):
            for r in (1, 2, 3, 4):
                out.append((src, os.path.join(LIBDIR, '%s_r%d.o' % (base, r)), ['-DOFD_INST_R=%d' % r]))
        else:
            out.append((src, os.path.join(LIBDIR, base + '.o'), []))
    return out


def _newest_input():
    paths = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if not os.path.isdir(os.path.join(CSRC, f))]
    paths += [os.path.join(CSRC, 'generated', f) for f in os.listdir(os.path.join(CSRC, 'generated'))]
    paths += [os.path.join(INCLUDE, 'ofd.h')]
    return max(os.path.getmtime(p) for p in paths)


def up_to_date():
    return os.path.exists(LIBNAME) and os.path.getmtime(LIBNAME) >= _newest_input()


def build(force=False, verbose=False, extra_flags=()):
    """Compile csrc/*.cu and link lib/libofd.so; returns the library path."""
    if not force and up_to_date():
        return LIBNAME
    os.makedirs(LIBDIR, exist_ok=True)
    cc = nvcc()

    def compile_one(job):
        src, obj, defs = job
        cmd = [cc] + ARCH + NVCC_FLAGS + list(extra_flags) + defs + ['-I', INCLUDE, '-I', CSRC, '-c', src, '-o', obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError('nvcc failed for %s:\n%s\n%s' % (src, ' '.join(cmd), r.stderr[-6000:]))
        if verbose and r.stderr:
            print(r.stderr)
        return obj

    js = jobs()
    with ThreadPoolExecutor(max_workers=min(len(js), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, js))
    tmp = LIBNAME + '.tmp'
    cmd = [cc] + ARCH + ['-shared', '-o', tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError('nvcc link failed:\n%s\n%s' % (' '.join(cmd), r.stderr[-4000:]))
    os.replace(tmp, LIBNAME)
    return LIBNAME


if __name__ == '__main__':
    import sys
    print(build(force='--force' in sys.argv, verbose=True))
