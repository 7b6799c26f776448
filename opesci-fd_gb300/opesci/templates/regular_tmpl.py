"""CUDA program template of a RegularGrid (the acoustic scheme; the CUDA
counterpart of the reference's Regular3DTemplate,
opesci/templates/regular3d_tmpl.py:7-134, with the program blocks of
opesci/regulargrid.py:390-719).

The emitted .cu file keeps the reference's program blocks and C ABI:

  constants            dims, spacing, dt, ntsteps, time-level variables and
                       the parameters of the model (c, v)
  structs              extern "C" OpesciGrid / OpesciConvergence / OpesciProfiling
  initialisation       level 0 on the whole padded grid from the analytic
                       solution at t = 0, with the loop indices substituted for
                       the coordinates as the reference does, then level _t1
                       on the interior from the second-initialisation
                       expression (regulargrid.py:498-564); both printed with
                       the C printer and evaluated on the GPU in the same C
                       arithmetic (built with -fmad=false)
  time loop            the update expression as a term table for the device
                       runtime's regular sweep (ofd_regular_step), rotating
                       three levels like the reference (_t0 = _ti % 3)
  opesci_convergence   L2 error of level ntsteps % 2 against the analytic
                       solution at t = dt*ntsteps on the interior, coordinates
                       dx*(_x - margin) (regulargrid.py:650-700), in FP64 on
                       the GPU
  opesci_free, main    as in the reference

The update expression must be a sum of (literal x array) products, which is
what the reference's defaults produce (expand=True, eval_const=True).
"""
import re

import numpy as np

from ..codeprinter import ccode
from .cuda_gen import decimal_to_f32

__all__ = ['RegularCudaTemplate', 'model_terms', 'regular_terms', 'split_terms']

_COEF_FLOAT = re.compile(r'^(\d+\.\d*(?:e[+-]?\d+)?)F$')
_COEF_INT = re.compile(r'^(\d+)$')
_COEF_RAT = re.compile(r'^(\d+)\.0F/(\d+)\.0F$')


def split_terms(text):
    """Split a printed sum into (sign, term) pairs at top-level binary + and
    - (those outside brackets and parentheses, preceded by a space)."""
    terms = []
    depth = 0
    start = 0
    sign = 1
    i = 0
    if text.startswith('-'):
        sign, start, i = -1, 1, 1
    while i < len(text):
        ch = text[i]
        if ch in '[(':
            depth += 1
        elif ch in '])':
            depth -= 1
        elif depth == 0 and ch in '+-' and i >= 1 and text[i - 1] == ' ' and i + 1 < len(text) and text[i + 1] == ' ':
            terms.append((sign, text[start:i - 1].strip()))
            sign = 1 if ch == '+' else -1
            start = i + 2
            i += 1
        i += 1
    terms.append((sign, text[start:].strip()))
    return terms


def _coef_value(text):
    """float32 value of a printed coefficient as the C compiler forms it."""
    m = _COEF_FLOAT.match(text)
    if m:
        return decimal_to_f32(m.group(1))
    m = _COEF_INT.match(text)
    if m:
        return np.float32(int(m.group(1)))
    m = _COEF_RAT.match(text)
    if m:
        return np.float32(np.float32(int(m.group(1))) / np.float32(int(m.group(2))))
    raise ValueError('coefficient %r is not a literal' % text)


def model_terms(grid, field):
    """regular_terms of the grid's update; with the expand or eval_const
    switch off, of the same update in the default printed form
    (cuda_gen.default_form), which rounds differently from the reference's
    unexpanded or named-constant C by ~1e-7 relative."""
    if grid.expand and grid.eval_const:
        return regular_terms(grid, field)
    from .cuda_gen import default_form
    with default_form(grid):
        return regular_terms(grid, field)


def regular_terms(grid, field):
    """The update expression of ``field`` as the device runtime's term table:
    a list of (level, (dx, dy, dz), coef) in the order of the printed C sum,
    level 1 for time level _t1 (t) and 0 for _t0 (t-1); coef is the float32
    value of the signed literal.  Raises ValueError when the expression is
    not a sum of literal x array products."""
    if not (grid.expand and grid.eval_const):
        raise ValueError('the device sweep needs the expanded, constant-folded update expression '
                         '(expand=True, eval_const=True)')
    grid.create_const_dict()
    text = ccode(grid.kernel_sympy(field))
    name = ccode(field.label)
    tnames = {grid.time[0].name: 0, grid.time[1].name: 1}
    idx_names = [str(i) for i in grid.index]
    arr = re.compile(r'^%s\[(\w+)\]' % re.escape(name) + ''.join(
        r'\[%s(?: ([+-]) (\d+))?\]' % re.escape(n) for n in idx_names) + '$')
    out = []
    for sign, term in split_terms(text):
        if '*' in term:
            ctext, atext = term.rsplit('*', 1)
        else:
            ctext, atext = '1', term
        m = arr.match(atext)
        if m is None:
            raise ValueError('term %r of %s is not a literal times an array of %s' % (term, name, name))
        g = m.groups()
        if g[0] not in tnames:
            raise ValueError('term %r reads time level %s' % (term, g[0]))
        off = []
        for k in range(len(idx_names)):
            s, v = g[1 + 2 * k], g[2 + 2 * k]
            off.append(0 if s is None else (int(v) if s == '+' else -int(v)))
        coef = _coef_value(ctext) * np.float32(sign)
        out.append((tnames[g[0]], tuple(off), float(coef)))
    return out


def _lit(v):
    return repr(float(v))


class RegularCudaTemplate(object):
    """Emits the CUDA program of a solved RegularGrid."""

    def __init__(self, grid):
        self.grid = grid

    def generate(self):
        g = self.grid
        if len(g.fields) != 1:
            raise NotImplementedError('the regular-grid device runtime advances one field')
        f = g.fields[0]
        name = ccode(f.label)
        real = g.real_t
        storage = 'OFD_F64' if g.double else 'OFD_F32'
        terms = model_terms(g, f)
        init1 = ccode(g.initial_kernel(f))
        init2 = ccode(g.second_initial_kernel(f))
        sol = getattr(f, 'sol', None)
        vol = 1.0
        for sp in g.spacing:
            vol *= sp.value
        m = g.margin.value
        L = []
        A = L.append
        A('// Generated by opesci (RegularCudaTemplate): regular-grid scheme, order %s,' % (g.order,))
        A('// grid %s, %d steps.' % ([d.value for d in g.dim], g.ntsteps.value))
        for inc in ('cstdio', 'cstdlib', 'cstring', 'cmath', 'string', 'vector', 'cuda_runtime.h'):
            A('#include <%s>' % inc)
        A('#include "ofd.h"')
        A('')
        A('typedef %s real_t;' % real)
        A('#define OFD_TRY(call) do { int _r = (call); if (_r) { fprintf(stderr, "%s: %s\\n", #call, ofd_last_error()); return _r; } } while (0)')
        A('#define CU_TRY(call) do { cudaError_t _e = (call); if (_e != cudaSuccess) { fprintf(stderr, "%s: %s\\n", #call, cudaGetErrorString(_e)); return -2; } } while (0)')
        A('')
        for k, d in enumerate(g.dim):
            A('constexpr int n%d = %d;' % (k + 1, d.value))
        A('constexpr int margin = %d;' % m)
        A('constexpr int ntsteps = %d;' % g.ntsteps.value)
        # each constant with its own C type, as the reference declares them
        # (regulargrid.py:390-406): dt keeps the type it was created with
        A('[[maybe_unused]] constexpr %s dt = %s;' % (g.dt.type, _lit(g.dt.value)))
        for sp in g.spacing:
            A('[[maybe_unused]] constexpr %s %s = %s;' % (sp.type, sp.name, _lit(sp.value)))
        for v in g.defined_variable.values():
            if v.constant:
                A('[[maybe_unused]] constexpr %s %s = %s;' % (v.type, v.name, _lit(v.value)))
        # time-level variables hold their initial values during the
        # initialisation
        for tv in g.time:
            A('[[maybe_unused]] constexpr int %s = %d;' % (tv.name, tv.value))
        A('')
        A('static const int term_level[%d] = {%s};' % (len(terms), ', '.join(str(t[0]) for t in terms)))
        A('static const int term_offset[%d][3] = {%s};' % (len(terms), ', '.join(
            '{%d, %d, %d}' % t[1] for t in terms)))
        A('static const double term_coef[%d] = {%s};' % (len(terms), ', '.join(_lit(t[2]) for t in terms)))
        A('')
        A('extern "C" struct OpesciGrid { real_t *%s; };' % name)
        A('extern "C" struct OpesciConvergence { real_t %s_l2; };' % name)
        papi = ''.join(' long long g_%s;' % e for e in getattr(g, '_papi_events', []))
        A('extern "C" struct OpesciProfiling { float g_rtime; float g_ptime; float g_mflops;%s };' % papi)
        A('')
        A('typedef real_t (*levels_t)[n1][n2][n3];')
        A('')
        A('// level 0 on the whole padded grid (regulargrid.py:498-534)')
        A('__global__ void first_init(real_t *buf) {')
        A('  levels_t %s = (levels_t)buf;' % name)
        A('  const long n = (long)n1 * n2 * n3;')
        A('  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {')
        A('    const int _z = (int)(i % n3); const long r = i / n3; const int _y = (int)(r % n2); const int _x = (int)(r / n2);')
        A('    (void)_x; (void)_y; (void)_z;')
        A('    %s[0][_x][_y][_z] = %s;' % (name, init1))
        A('  }')
        A('}')
        A('')
        A('// level _t1 on the interior from level _t0 (regulargrid.py:536-564)')
        A('__global__ void second_init(real_t *buf) {')
        A('  levels_t %s = (levels_t)buf;' % name)
        A('  const long n = (long)n1 * n2 * n3;')
        A('  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {')
        A('    const int _z = (int)(i % n3); const long r = i / n3; const int _y = (int)(r % n2); const int _x = (int)(r / n2);')
        A('    if (_x < margin || _x >= n1 - margin || _y < margin || _y >= n2 - margin || _z < margin || _z >= n3 - margin) continue;')
        A('    %s[%s][_x][_y][_z] = %s;' % (name, g.time[1].name, init2))
        A('  }')
        A('}')
        A('')
        if sol is not None:
            A('__device__ double sol_at(real_t x, real_t y, real_t z, double _t) {')
            A('  (void)x; (void)y; (void)z; (void)_t;')
            A('  return %s;' % ccode(sol))
            A('}')
            A('')
            A('// FP64 squared error against the analytic solution, one partial per block;')
            A('// coordinates as `real_t x = dx1*(_x - margin)` (regulargrid.py:678-682)')
            A('__global__ void l2_partial(const real_t *fld, double t, double *partial) {')
            A('  const long n = (long)n1 * n2 * n3;')
            A('  double acc = 0.0;')
            A('  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {')
            A('    const int _z = (int)(i % n3); const long r = i / n3; const int _y = (int)(r % n2); const int _x = (int)(r / n2);')
            A('    if (_x < margin || _x >= n1 - margin || _y < margin || _y >= n2 - margin || _z < margin || _z >= n3 - margin) continue;')
            A('    const real_t x = %s*(_x - margin), y = %s*(_y - margin), z = %s*(_z - margin);'
              % tuple(sp.name for sp in g.spacing))
            A('    const double e = (double)fld[i] - sol_at(x, y, z, t);')
            A('    acc += e * e;')
            A('  }')
            A('  __shared__ double sh[256];')
            A('  sh[threadIdx.x] = acc;')
            A('  __syncthreads();')
            A('  for (int w = 128; w > 0; w >>= 1) { if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w]; __syncthreads(); }')
            A('  if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];')
            A('}')
            A('')
        A('static ofd_regular *g_handle = nullptr;')
        A('')
        A('extern "C" int opesci_execute(OpesciGrid *grid, OpesciProfiling *profiling) {')
        A('  const long n = (long)n1 * n2 * n3;')
        A('  ofd_regular_config cfg;')
        A('  memset(&cfg, 0, sizeof(cfg));')
        A('  cfg.dim[0] = n1; cfg.dim[1] = n2; cfg.dim[2] = n3;')
        A('  cfg.margin = margin;')
        A('  cfg.storage = %s;' % storage)
        A('  cfg.nterms = %d;' % len(terms))
        A('  for (int k = 0; k < %d; ++k) {' % len(terms))
        A('    cfg.level[k] = term_level[k]; cfg.coef[k] = term_coef[k];')
        A('    for (int d = 0; d < 3; ++d) cfg.offset[k][d] = term_offset[k][d];')
        A('  }')
        A('  if (g_handle) { ofd_regular_destroy(g_handle); g_handle = nullptr; }')
        A('  OFD_TRY(ofd_regular_create(&cfg, &g_handle));')
        A('  cudaStream_t st = (cudaStream_t)ofd_regular_stream(g_handle);')
        A('  real_t *buf = nullptr;')
        A('  CU_TRY(cudaMallocAsync((void **)&buf, sizeof(real_t) * 3 * n, st));')
        A('  CU_TRY(cudaMemsetAsync(buf, 0, sizeof(real_t) * 3 * n, st));')
        A('  first_init<<<1216, 256, 0, st>>>(buf);')
        A('  second_init<<<1216, 256, 0, st>>>(buf);')
        A('  CU_TRY(cudaGetLastError());')
        A('  for (int l = 0; l < 3; ++l) OFD_TRY(ofd_regular_upload_device(g_handle, l, buf + l * n));')
        A('  cudaEvent_t e0, e1;')
        A('  cudaEventCreate(&e0); cudaEventCreate(&e1);')
        A('  cudaEventRecord(e0, st);')
        if g.output_vts:
            # the output_vts step after every time step (regulargrid.py:702-719):
            # the new level _t2 = (_ti + 2) % 3 to <field>_<ti>.vts with the
            # reference's margin argument of 2, as float values
            sp = [s.name for s in g.spacing]
            A('  {')
            A('    std::vector<real_t> vts_raw(n);')
            A('    std::vector<float> vts_buf(n);')
            A('    const int vts_dims[3] = {n1, n2, n3};')
            A('    const float vts_spacing[3] = {(float)%s, (float)%s, (float)%s};' % tuple(sp))
            A('    for (int _ti = 0; _ti < ntsteps; ++_ti) {')
            A('      OFD_TRY(ofd_regular_step(g_handle, 1));')
            A('      OFD_TRY(ofd_regular_download(g_handle, (_ti + 2) % 3, vts_raw.data()));')
            A('      for (long i = 0; i < n; ++i) vts_buf[i] = (float)vts_raw[i];')
            A('      const std::string vtkfile = "%s_" + std::to_string(_ti);' % name)
            A('      OFD_TRY(ofd_write_field_vts_3d(vtkfile.c_str(), vts_dims, vts_spacing, 2, vts_buf.data()));')
            A('    }')
            A('  }')
        else:
            A('  OFD_TRY(ofd_regular_step(g_handle, ntsteps));')
        A('  cudaEventRecord(e1, st);')
        A('  OFD_TRY(ofd_regular_sync(g_handle));')
        A('  float ms = 0.f;')
        A('  cudaEventElapsedTime(&ms, e0, e1);')
        A('  cudaEventDestroy(e0); cudaEventDestroy(e1);')
        A('  profiling->g_rtime = ms / 1000.0f; profiling->g_ptime = ms / 1000.0f; profiling->g_mflops = 0.0f;')
        for e in getattr(g, '_papi_events', []):
            A('  profiling->g_%s = 0;' % e)
        if g.profiling:
            # one multiplication per term and one addition per term after the
            # first, per interior point, over the timed loop
            A('  {')
            A('    const double pts = (double)(n1 - 2 * margin) * (n2 - 2 * margin) * (n3 - 2 * margin);')
            A('    if (ms > 0.f) profiling->g_mflops = (float)(%d.0 * pts * ntsteps / (ms / 1000.0) / 1e6);'
              % (2 * len(terms) - 1))
            A('  }')
        A('  void *p = nullptr;')
        A('  if (posix_memalign(&p, 4096, sizeof(real_t) * 3 * n)) return -3;')
        A('  grid->%s = (real_t *)p;' % name)
        A('  for (int l = 0; l < 3; ++l) OFD_TRY(ofd_regular_download(g_handle, l, (real_t *)p + l * n));')
        A('  CU_TRY(cudaFreeAsync(buf, st));')
        A('  OFD_TRY(ofd_regular_sync(g_handle));')
        A('  return 0;')
        A('}')
        A('')
        A('extern "C" int opesci_convergence(OpesciGrid *grid, OpesciConvergence *conv) {')
        A('  (void)grid;')
        A('  conv->%s_l2 = 0;' % name)
        if sol is not None:
            A('  if (!g_handle) return -4;')
            A('  const long n = (long)n1 * n2 * n3;')
            A('  cudaStream_t st = (cudaStream_t)ofd_regular_stream(g_handle);')
            A('  real_t *tmp = nullptr; double *part = nullptr;')
            A('  CU_TRY(cudaMalloc((void **)&tmp, sizeof(real_t) * n));')
            A('  CU_TRY(cudaMalloc((void **)&part, sizeof(double) * 1024));')
            # the reference reads level ntsteps % 2 of its three levels
            A('  OFD_TRY(ofd_regular_download_device(g_handle, %d, tmp));' % (g.ntsteps.value % 2))
            A('  l2_partial<<<1024, 256, 0, st>>>(tmp, %s, part);' % _lit(g.dt.value * g.ntsteps.value))
            A('  std::vector<double> hp(1024);')
            A('  CU_TRY(cudaMemcpyAsync(hp.data(), part, sizeof(double) * 1024, cudaMemcpyDeviceToHost, st));')
            A('  CU_TRY(cudaStreamSynchronize(st));')
            A('  double s = 0.0;')
            A('  for (int i = 0; i < 1024; ++i) s += hp[i];')
            A('  conv->%s_l2 = (real_t)sqrt(s * %r);' % (name, vol))
            A('  cudaFree(tmp); cudaFree(part);')
        A('  return 0;')
        A('}')
        A('')
        A('extern "C" int opesci_free(OpesciGrid *grid) {')
        A('  free(grid->%s); grid->%s = nullptr;' % (name, name))
        A('  if (g_handle) { ofd_regular_destroy(g_handle); g_handle = nullptr; }')
        A('  return 0;')
        A('}')
        A('')
        A('int main() {')
        A('  OpesciGrid grid; OpesciConvergence conv; OpesciProfiling profiling;')
        A('  if (opesci_execute(&grid, &profiling)) return 1;')
        A('  if (opesci_convergence(&grid, &conv)) return 1;')
        A('  opesci_free(&grid);')
        A('  printf("%s_l2\\t%%.10f\\n", conv.%s_l2);' % (name, name))
        A('  return 0;')
        A('}')
        return '\n'.join(L) + '\n'
