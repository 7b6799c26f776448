"""CUDA program template of a StaggeredGrid (the CUDA counterpart of the
reference's Staggered3DTemplate, opesci/templates/staggered3d_tmpl.py and
regular3d_tmpl.py:7-134).

The emitted .cu file keeps the reference's program blocks and C ABI:

  constants            the model's dims, spacing, dt, ntsteps, media constants
                       and the literal tables of its generated update
                       expressions (opesci/templates/cuda_gen.py)
  structs              extern "C" OpesciGrid / OpesciConvergence / OpesciProfiling
  analytic solutions   one __device__ function per field, printed from
                       field.sol with the C printer
  opesci_execute       device runtime handle, media, analytic initial state
                       (t = 0 for stresses, dt/2 for velocities, coordinates
                       rounded like the reference's `real_t x = dx1*(_x - m)`),
                       initial ghosts, the time loop (ofd_step, CUDA events),
                       and the final levels copied to host arrays published
                       through OpesciGrid
  opesci_convergence   L2 error against the analytic solution at the final
                       time, on the GPU, accumulated in FP64
  opesci_free, main    as in the reference
"""
from ..codeprinter import ccode

__all__ = ['StaggeredCudaTemplate']

_FACE_NAMES = {'levander': 'OFD_BC_LEVANDER', 'robertsson': 'OFD_BC_ROBERTSSON'}


def _lit(v):
    r = repr(float(v))
    return r


class StaggeredCudaTemplate(object):
    """Emits the CUDA program of a solved StaggeredGrid."""

    def __init__(self, grid):
        self.grid = grid

    # ------------------------------------------------------------ pieces
    def _constants(self):
        g = self.grid
        out = []
        # the reference names these dim1..dim3; dim3 is a CUDA type, so the
        # CUDA program calls them n1..n3
        for k, d in enumerate(g.dim):
            out.append('constexpr int n%d = %d;' % (k + 1, d.value))
        out.append('constexpr int margin = %d;' % g.margin.value)
        out.append('constexpr int ntsteps = %d;' % g.ntsteps.value)
        out.append('constexpr real_t dt = %s;' % _lit(g.dt.value))
        for sp in g.spacing:
            out.append('constexpr real_t %s = %s;' % (sp.name, _lit(sp.value)))
        for v in g.defined_variable.values():
            if v.constant:
                out.append('constexpr real_t %s = %s;' % (v.name, _lit(v.value)))
        return out

    def _tables(self):
        from . import cuda_gen
        g = self.grid
        # with the expand or eval_const switch off, the same update in the
        # default printed form (cuda_gen.default_form)
        tabs, _ = cuda_gen.model_tables(g)
        key = 'so%d_%s' % (g.order[1], 'het' if g.read else 'const')
        pre = cuda_gen.prebuilt_signatures().get(key)
        if pre is None or pre['stress'] != tabs['stress'][0] or pre['velocity'] != tabs['velocity'][0]:
            raise ValueError('the update expressions of this model (%s) do not match the prebuilt CUDA '
                             'expressions of libofd: the device kernels are built for the velocity-stress '
                             'equations' % key)
        ks, kv = tabs['stress'][1], tabs['velocity'][1]
        fmt = lambda a: ', '.join('%sf' % repr(float(x)) for x in a)  # noqa: E731
        out = ['static const float ofd_ks[%d] = {%s};' % (len(ks), fmt(ks)),
               'static const float ofd_kv[%d] = {%s};' % (len(kv), fmt(kv)),
               'constexpr int ofd_het = %d;' % (1 if g.read else 0)]
        # space order 4 with Levander faces: the printed ghost equations' literal
        # table, when their structure is the prebuilt one (not for FP64 storage)
        gt = None if g.double else cuda_gen.model_ghost_table(g)
        if gt is not None and pre.get('ghost') == gt[0]:
            out.append('static const float ofd_kg[%d] = {%s};' % (len(gt[1]), fmt(gt[1])))
            self._nkg = len(gt[1])
        else:
            self._nkg = 0
        return out, len(ks), len(kv)

    def _flops_per_point(self):
        """Additions plus multiplications of the nine update expressions."""
        g = self.grid
        v, s = g.get_velocity_kernel_ai(), g.get_stress_kernel_ai()
        return int(v[2] + v[3] + s[2] + s[3])

    def _solutions(self):
        g = self.grid
        out = []
        cases = []
        for i, f in enumerate(g.fields):
            sol = getattr(f, 'sol', None)
            name = ccode(f.label)
            if sol is None:
                continue
            expr = ccode(sol)
            out.append('__device__ double sol_%s(real_t x, real_t y, real_t z, double _t) {' % name)
            out.append('  (void)x; (void)y; (void)z; (void)_t;')
            out.append('  return %s;' % expr)
            out.append('}')
            cases.append('    case %d: return sol_%s(x, y, z, t);' % (i, name))
        out.append('__device__ double sol_field(int f, real_t x, real_t y, real_t z, double t) {')
        out.append('  switch (f) {')
        out += cases
        out.append('  }')
        out.append('  return 0.0;')
        out.append('}')
        return out

    def generate(self):
        g = self.grid
        names = [ccode(f.label) for f in g.fields]
        has_sol = [getattr(f, 'sol', None) is not None for f in g.fields]
        stag = [[1 if f.staggered[d + 1] else 0 for d in range(3)] for f in g.fields]
        tstag = [1 if f.staggered[0] else 0 for f in g.fields]
        faces = ['OFD_BC_NONE'] * 6
        for (dim, side), algo in getattr(g, 'free_surface', {}).items():
            faces[2 * (dim - 1) + side] = _FACE_NAMES[algo]
        tables, nks, nkv = self._tables()
        weights = g.fd_weights() + [0.0] * (4 - len(g.fd_weights()))
        vol = 1.0
        for sp in g.spacing:
            vol *= sp.value
        L = []
        A = L.append
        A('// Generated by opesci (StaggeredCudaTemplate): elastic velocity-stress model,')
        A('// space order %d, grid %s, %d steps, %s media.' % (g.order[1], [d.value for d in g.dim],
                                                              g.ntsteps.value, 'file' if g.read else 'constant'))
        A('#include <cstdio>')
        A('#include <cstdlib>')
        A('#include <cstring>')
        A('#include <cmath>')
        A('#include <string>')
        A('#include <vector>')
        A('#include <cuda_runtime.h>')
        A('#include "ofd.h"')
        A('')
        A('typedef %s real_t;' % ('double' if g.double else 'float'))
        A('#define OFD_TRY(call) do { int _r = (call); if (_r) { fprintf(stderr, "%s: %s\\n", #call, ofd_last_error()); return _r; } } while (0)')
        A('#define CU_TRY(call) do { cudaError_t _e = (call); if (_e != cudaSuccess) { fprintf(stderr, "%s: %s\\n", #call, cudaGetErrorString(_e)); return -2; } } while (0)')
        A('')
        L.extend(self._constants())
        L.extend(tables)
        A('static const int field_has_sol[9] = {%s};' % ', '.join(str(int(x)) for x in has_sol))
        A('static const int field_stag[9][3] = {%s};' % ', '.join('{%d, %d, %d}' % tuple(s) for s in stag))
        A('static const int field_tstag[9] = {%s};' % ', '.join(str(x) for x in tstag))
        if g.source is not None:
            (sx, sy, sz), wav = g.source
            sigs = list(wav) if isinstance(wav, tuple) else [wav]
            A('static const int src_pos[3] = {%d, %d, %d};' % (sx, sy, sz))
            A('static const float src_wav[%d][%d] = {%s};' % (
                len(sigs), len(sigs[0]),
                ', '.join('{%s}' % ', '.join('%sf' % repr(float(w)) for w in sig) for sig in sigs)))
        A('')
        A('extern "C" struct OpesciGrid { %s };' % ' '.join('real_t *%s;' % n for n in names))
        A('extern "C" struct OpesciConvergence { %s };' % ' '.join('real_t %s_l2;' % n for n in names))
        # PAPI event slots (regulargrid.py:350-354): kept for the struct layout
        # the caller defines; hardware counters of the host CPU have no meaning
        # for a GPU run and stay zero
        papi = ''.join(' long long g_%s;' % e for e in getattr(g, '_papi_events', []))
        A('extern "C" struct OpesciProfiling { float g_rtime; float g_ptime; float g_mflops;%s };' % papi)
        A('')
        L.extend(self._solutions())
        A('')
        A('// coordinate of index i on an axis with spacing h, staggered by s/2,')
        A('// rounded like `real_t x = dx1*(_x - m)` (staggeredgrid.py:632-641)')
        A('__device__ __forceinline__ real_t coord(real_t h, int i, int s) {')
        A('  return (real_t)((double)h * ((double)(i - margin) + 0.5 * s));')
        A('}')
        A('')
        A('// analytic value of field f at time t on its own index range, reference layout')
        A('__global__ void init_field(real_t *out, int f, int s0, int s1, int s2, double t) {')
        A('  const long n = (long)n1 * n2 * n3;')
        A('  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {')
        A('    const int z = (int)(i % n3); const long r = i / n3; const int y = (int)(r % n2); const int x = (int)(r / n2);')
        A('    const bool in = x >= margin && x < n1 - margin - s0 && y >= margin && y < n2 - margin - s1 &&')
        A('                    z >= margin && z < n3 - margin - s2;')
        A('    out[i] = in ? (real_t)sol_field(f, coord(dx1, x, s0), coord(dx2, y, s1), coord(dx3, z, s2), t) : (real_t)0;')
        A('  }')
        A('}')
        A('')
        A('// FP64 squared error against the analytic solution, one partial per block')
        A('__global__ void l2_partial(const real_t *fld, int f, int s0, int s1, int s2, double t, double *partial) {')
        A('  const long n = (long)n1 * n2 * n3;')
        A('  double acc = 0.0;')
        A('  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {')
        A('    const int z = (int)(i % n3); const long r = i / n3; const int y = (int)(r % n2); const int x = (int)(r / n2);')
        A('    if (x >= margin && x < n1 - margin - s0 && y >= margin && y < n2 - margin - s1 &&')
        A('        z >= margin && z < n3 - margin - s2) {')
        A('      const double e = (double)fld[i] - sol_field(f, coord(dx1, x, s0), coord(dx2, y, s1), coord(dx3, z, s2), t);')
        A('      acc += e * e;')
        A('    }')
        A('  }')
        A('  __shared__ double sh[256];')
        A('  sh[threadIdx.x] = acc;')
        A('  __syncthreads();')
        A('  for (int w = 128; w > 0; w >>= 1) { if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w]; __syncthreads(); }')
        A('  if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];')
        A('}')
        A('')
        A('static ofd_handle *g_handle = nullptr;')
        A('')
        A('static int read_raw(const char *path, std::vector<float> &v) {')
        A('  FILE *fp = fopen(path, "rb");')
        A('  if (!fp) { fprintf(stderr, "cannot open %s\\n", path); return -1; }')
        A('  const size_t got = fread(v.data(), sizeof(float), v.size(), fp);')
        A('  fclose(fp);')
        A('  return got == v.size() ? 0 : -1;')
        A('}')
        A('')
        A('extern "C" int opesci_execute(OpesciGrid *grid, OpesciProfiling *profiling) {')
        A('  const long n = (long)n1 * n2 * n3;')
        A('  ofd_config cfg;')
        A('  memset(&cfg, 0, sizeof(cfg));')
        A('  cfg.dim[0] = n1; cfg.dim[1] = n2; cfg.dim[2] = n3;')
        A('  cfg.space_order = %d;' % g.order[1])
        A('  cfg.storage = %s;' % ('OFD_F64' if g.double else 'OFD_F32'))
        A('  cfg.legacy_bc = %d;' % (1 if getattr(g, 'legacy_bc', False) else 0))
        for i, fc in enumerate(faces):
            A('  cfg.free_surface[%d] = %s;' % (i, fc))
        A('  cfg.spacing[0] = dx1; cfg.spacing[1] = dx2; cfg.spacing[2] = dx3;')
        A('  cfg.dt = dt;')
        for k in range(4):
            A('  cfg.weights[%d] = %s;' % (k, _lit(weights[k])))
        A('  for (int f = 0; f < 9; ++f) cfg.field_scale[f] = 1.0f;')
        A('  if (g_handle) { ofd_destroy(g_handle); g_handle = nullptr; }')
        A('  OFD_TRY(ofd_create(&cfg, &g_handle));')
        A('  OFD_TRY(ofd_set_coefficients(g_handle, ofd_het, ofd_ks, %d, ofd_kv, %d));' % (nks, nkv))
        if self._nkg:
            A('  OFD_TRY(ofd_set_ghost_coefficients(g_handle, ofd_het, ofd_kg, %d));' % self._nkg)
        if g.read:
            A('  {')
            A('    std::vector<float> rho_a(n), vp_a(n), vs_a(n);')
            A('    if (read_raw("%s", rho_a) || read_raw("%s", vp_a) || read_raw("%s", vs_a)) return -1;'
              % (g.rho_file, g.vp_file, g.vs_file))
            A('    OFD_TRY(ofd_set_media(g_handle, rho_a.data(), vp_a.data(), vs_a.data()));')
            A('  }')
        else:
            A('  OFD_TRY(ofd_set_media_const(g_handle, beta, lambda, mu));')
        A('  real_t *tmp = nullptr;')
        A('  CU_TRY(cudaMalloc((void **)&tmp, sizeof(real_t) * n));')
        A('  cudaStream_t st = (cudaStream_t)ofd_stream(g_handle);')
        if g.double:
            A('  std::vector<double> init_host(n);')
        A('  for (int f = 0; f < 9; ++f) {')
        A('    if (!field_has_sol[f]) continue;')
        A('    const double t0 = field_tstag[f] ? dt / 2 : 0.0;')
        A('    init_field<<<1216, 256, 0, st>>>(tmp, f, field_stag[f][0], field_stag[f][1], field_stag[f][2], t0);')
        if g.double:
            # FP64 storage takes double host arrays: the initial level goes
            # through the host once, exactly
            A('    CU_TRY(cudaMemcpyAsync(init_host.data(), tmp, sizeof(double) * n, cudaMemcpyDeviceToHost, st));')
            A('    CU_TRY(cudaStreamSynchronize(st));')
            A('    OFD_TRY(ofd_upload_field_f64(g_handle, f, 0, init_host.data()));')
        else:
            A('    OFD_TRY(ofd_upload_field_device(g_handle, f, 0, tmp));')
        A('  }')
        A('  OFD_TRY(ofd_apply_boundary_init(g_handle, 0));')
        if g.source is not None:
            if isinstance(g.source[1], tuple):
                A('  OFD_TRY(ofd_set_source_xyz(g_handle, src_pos[0], src_pos[1], src_pos[2], src_wav[0], src_wav[1], '
                  'src_wav[2], %d));' % len(g.source[1][0]))
            else:
                A('  OFD_TRY(ofd_set_source(g_handle, src_pos[0], src_pos[1], src_pos[2], src_wav[0], %d));'
                  % len(g.source[1]))
        A('  OFD_TRY(ofd_sync(g_handle));')
        A('  cudaEvent_t e0, e1;')
        A('  cudaEventCreate(&e0); cudaEventCreate(&e1);')
        A('  cudaEventRecord(e0, st);')
        if g.output_vts:
            # the output_vts step after every time step (staggered3d_tmpl.py:56-58,
            # regulargrid.py:702-719): U of the new level to U_<ti>.vts with the
            # reference's margin argument of 2; its dims {dim1, dim1, dim1} are
            # the grid's for cubic grids, which are the only ones it writes whole
            A('  {')
            A('    std::vector<float> vts_buf(n);')
            A('    const int vts_dims[3] = {n1, n2, n3};')
            A('    const float vts_spacing[3] = {dx1, dx2, dx3};')
            A('    for (int _ti = 0; _ti < ntsteps; ++_ti) {')
            A('      OFD_TRY(ofd_step(g_handle, 1));')
            A('      OFD_TRY(ofd_download_field(g_handle, 0, (_ti + 1) % 2, vts_buf.data()));')
            A('      const std::string vtkfile = "U_" + std::to_string(_ti);')
            A('      OFD_TRY(ofd_write_field_vts_3d(vtkfile.c_str(), vts_dims, vts_spacing, 2, vts_buf.data()));')
            A('    }')
            A('  }')
        else:
            A('  OFD_TRY(ofd_step(g_handle, ntsteps));')
        A('  cudaEventRecord(e1, st);')
        A('  OFD_TRY(ofd_sync(g_handle));')
        A('  float ms = 0.f;')
        A('  cudaEventElapsedTime(&ms, e0, e1);')
        A('  cudaEventDestroy(e0); cudaEventDestroy(e1);')
        A('  profiling->g_rtime = ms / 1000.0f; profiling->g_ptime = ms / 1000.0f; profiling->g_mflops = 0.0f;')
        for e in getattr(g, '_papi_events', []):
            A('  profiling->g_%s = 0;' % e)
        if g.profiling:
            # the update expressions' additions and multiplications per interior
            # point (get_kernel_ai's counts, regulargrid.py:293-327) over the timed loop
            fl = self._flops_per_point()
            A('  {')
            A('    const double pts = (double)(n1 - 2 * margin) * (n2 - 2 * margin) * (n3 - 2 * margin);')
            A('    if (ms > 0.f) profiling->g_mflops = (float)(%d.0 * pts * ntsteps / (ms / 1000.0) / 1e6);' % fl)
            A('  }')
        A('  real_t **dst[9] = {%s};' % ', '.join('&grid->%s' % nm for nm in names))
        A('  for (int f = 0; f < 9; ++f) {')
        A('    void *p = nullptr;')
        A('    if (posix_memalign(&p, 4096, sizeof(real_t) * 2 * n)) return -3;')
        A('    *dst[f] = (real_t *)p;')
        if g.double:
            A('    for (int l = 0; l < 2; ++l) OFD_TRY(ofd_download_field_f64(g_handle, f, l, (double *)p + l * n));')
        else:
            A('    for (int l = 0; l < 2; ++l) OFD_TRY(ofd_download_field(g_handle, f, l, (float *)p + l * n));')
        A('  }')
        A('  cudaFree(tmp);')
        A('  return 0;')
        A('}')
        A('')
        A('extern "C" int opesci_convergence(OpesciGrid *grid, OpesciConvergence *conv) {')
        A('  (void)grid;')
        A('  if (!g_handle) return -4;')
        A('  const long n = (long)n1 * n2 * n3;')
        A('  const int level = ntsteps % 2;')
        A('  real_t *out[9] = {%s};' % ', '.join('&conv->%s_l2' % nm for nm in names))
        A('  real_t *tmp = nullptr; double *part = nullptr;')
        A('  CU_TRY(cudaMalloc((void **)&tmp, sizeof(real_t) * n));')
        A('  CU_TRY(cudaMalloc((void **)&part, sizeof(double) * 1024));')
        A('  cudaStream_t st = (cudaStream_t)ofd_stream(g_handle);')
        A('  std::vector<double> hp(1024);')
        A('  for (int f = 0; f < 9; ++f) {')
        A('    *out[f] = 0;')
        A('    if (!field_has_sol[f]) continue;')
        A('    const double tn = dt * ntsteps + (field_tstag[f] ? dt / 2.0 : 0.0);')
        if g.double:
            # the published double arrays of opesci_execute, level ntsteps % 2
            A('    real_t *pub[9] = {%s};' % ', '.join('grid->%s' % nm for nm in names))
            A('    CU_TRY(cudaMemcpyAsync(tmp, pub[f] + (size_t)level * n, sizeof(double) * n, cudaMemcpyHostToDevice, st));')
        else:
            A('    OFD_TRY(ofd_download_field_device(g_handle, f, level, tmp));')
        A('    l2_partial<<<1024, 256, 0, st>>>(tmp, f, field_stag[f][0], field_stag[f][1], field_stag[f][2], tn, part);')
        A('    CU_TRY(cudaMemcpyAsync(hp.data(), part, sizeof(double) * 1024, cudaMemcpyDeviceToHost, st));')
        A('    CU_TRY(cudaStreamSynchronize(st));')
        A('    double s = 0.0;')
        A('    for (int i = 0; i < 1024; ++i) s += hp[i];')
        A('    *out[f] = (real_t)sqrt(s * %r);' % vol)
        A('  }')
        A('  cudaFree(tmp); cudaFree(part);')
        A('  return 0;')
        A('}')
        A('')
        A('extern "C" int opesci_free(OpesciGrid *grid) {')
        for nm in names:
            A('  free(grid->%s); grid->%s = nullptr;' % (nm, nm))
        A('  if (g_handle) { ofd_destroy(g_handle); g_handle = nullptr; }')
        A('  return 0;')
        A('}')
        A('')
        A('int main() {')
        A('  OpesciGrid grid; OpesciConvergence conv; OpesciProfiling profiling;')
        A('  if (opesci_execute(&grid, &profiling)) return 1;')
        A('  if (opesci_convergence(&grid, &conv)) return 1;')
        A('  opesci_free(&grid);')
        for f, hs in zip(g.fields, has_sol):
            if hs:
                nm = ccode(f.label)
                A('  printf("%s_l2\\t%%.10f\\n", conv.%s_l2);' % (nm, nm))
        A('  return 0;')
        A('}')
        return '\n'.join(L) + '\n'
