// Device runtime of the opesci-fd elastic hot path: handle lifecycle, HBM
// layout, media preprocessing, transfers and the time loop, exported through
// the C ABI of include/ofd.h.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <cstdarg>
#include <string>
#include <vector>

#include <cuda.h>
#include <mutex>

#include "ofd.h"
#include "ofd_impl.cuh"

namespace ofd {

static thread_local std::string g_last_error;

static int fail(int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

// for the other translation units of the library
int fail_msg(int code, const char *msg) { return fail(code, "%s", msg); }

#define OFD_CUDA(call)                                                                   \
  do {                                                                                   \
    cudaError_t _e = (call);                                                             \
    if (_e != cudaSuccess)                                                               \
      return fail(OFD_ECUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(_e),     \
                  __FILE__, __LINE__);                                                   \
  } while (0)

// Media preprocessing (staggeredgrid.py:571-597), evaluated in double and
// rounded to float like the reference's C expressions, on the whole padded
// grid with upper neighbours clamped at the last index: beta = 1/rho,
// lambda = rho (vp^2 - 2 vs^2), mu = rho vs^2; beta1..3 the means of beta and
// its upper neighbour along x/y/z; mu12/13/23 the harmonic means of mu over
// the four points of the cell edge (1/mu in double).  Two passes over a 3D
// grid of (z, y) blocks per x plane (no index divisions): the point values,
// then the averages.  FP64 division is the cost on this GPU (its FP64 rate is
// a small fraction of FP32), so each 1/mu is computed once per point and
// beta as a float division: (float)(1.0/(double)rho) equals the correctly
// rounded float quotient 1.0f/rho, since rounding a quotient of 24-bit
// operands first to 53 bits and then to 24 bits is innocuous (53 >= 2*24+2;
// S. A. Figueroa, "When is double rounding innocuous?", SIGNUM 1995).
__global__ void media_point_kernel(const float *__restrict__ rho, const float *__restrict__ vp,
                                   const float *__restrict__ vs, Geom g, float *o_beta, float *o_lam, float *o_mu,
                                   double *inv_mu, int x0) {
  const int z = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int x = x0 + (int)blockIdx.z;
  if (z >= g.n3 || y >= g.n2) return;
  const long i = ((long)x * g.n2 + y) * g.n3 + z;
  const long o = (long)x * g.plane + (long)y * g.P + z;
  const float rf = rho[i];
  const double r = rf, p = vp[i], s = vs[i];
  o_beta[o] = __fdiv_rn(1.0f, rf);
  o_lam[o] = (float)(r * (p * p - 2.0 * (s * s)));
  const float m = (float)(r * (s * s));
  o_mu[o] = m;
  inv_mu[i] = 1.0 / (double)m;
}

__global__ void media_avg_kernel(const float *o_beta_in, const double *__restrict__ im, Geom g, float *o_mu12,
                                 float *o_mu13, float *o_mu23, float *o_b1, float *o_b2, float *o_b3, int x0) {
  const int z = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int x = x0 + (int)blockIdx.z;
  if (z >= g.n3 || y >= g.n2) return;
  const int x1 = x + 1 < g.n1 ? x + 1 : x, y1 = y + 1 < g.n2 ? y + 1 : y, z1 = z + 1 < g.n3 ? z + 1 : z;
  auto D = [&](int a, int b, int c) { return ((long)a * g.n2 + b) * g.n3 + c; };
  auto O = [&](int a, int b, int c) { return (long)a * g.plane + (long)b * g.P + c; };
  const long o = O(x, y, z);
  const float b0 = o_beta_in[o];
  o_b1[o] = (b0 + o_beta_in[O(x1, y, z)]) * 0.5f;
  o_b2[o] = (b0 + o_beta_in[O(x, y1, z)]) * 0.5f;
  o_b3[o] = (b0 + o_beta_in[O(x, y, z1)]) * 0.5f;
  const double m0 = im[D(x, y, z)], mx = im[D(x1, y, z)], my = im[D(x, y1, z)], mz = im[D(x, y, z1)];
  o_mu12[o] = (float)(1.0 / (0.25 * (m0 + mx + my + im[D(x1, y1, z)])));
  o_mu13[o] = (float)(1.0 / (0.25 * (m0 + mx + mz + im[D(x1, y, z1)])));
  o_mu23[o] = (float)(1.0 / (0.25 * (m0 + my + mz + im[D(x, y1, z1)])));
}

// Library-owned stream-ordered pool for transient device scratch (media
// preprocessing, transfers of non-FP32 fields), one per device.  It keeps up
// to SCRATCH_KEEP bytes mapped between calls, so repeated jobs (serving,
// batching) do not map and unmap gigabytes per call; the device's default
// pool, which other libraries share, is left as it is.
constexpr unsigned long long SCRATCH_KEEP = 4ULL << 30;

cudaError_t scratch_alloc(void **p, size_t bytes, cudaStream_t st) {
  static std::mutex mu;
  static cudaMemPool_t pools[64] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaMallocAsync(p, bytes, st);
  cudaMemPool_t pool;
  {
    std::lock_guard<std::mutex> lock(mu);
    if (!pools[dev]) {
      cudaMemPoolProps props = {};
      props.allocType = cudaMemAllocationTypePinned;
      props.handleTypes = cudaMemHandleTypeNone;
      props.location.type = cudaMemLocationTypeDevice;
      props.location.id = dev;
      e = cudaMemPoolCreate(&pools[dev], &props);
      if (e != cudaSuccess) {
        pools[dev] = nullptr;
        return e;
      }
      unsigned long long keep = SCRATCH_KEEP;
      cudaMemPoolSetAttribute(pools[dev], cudaMemPoolAttrReleaseThreshold, &keep);
    }
    pool = pools[dev];
  }
  return cudaMallocFromPoolAsync(p, bytes, pool, st);
}

__global__ void fill_kernel(float *p, long n, float v) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) p[i] = v;
}

}  // namespace ofd

using namespace ofd;

struct ofd_handle {
  ofd_config cfg;
  DevState s;
  Backend *be = nullptr;
  cudaStream_t stream = nullptr;
  cudaStream_t copy_stream = nullptr;   // media uploads, overlapped with their preprocessing
  int device = 0;
  void *fields_raw = nullptr;   // one allocation for all fields
  void *media_raw = nullptr;    // one allocation for all media
  size_t field_bytes = 0, media_bytes = 0;
  long media_elems = 0;         // elements of one media array (padded)
  long level_elems = 0;         // elements of one field level (padded)
  long steps = 0;
  double *d_out = nullptr;      // 16 doubles
  int *d_err = nullptr;         // error word of bounded device waits
  TmaMaps *maps = nullptr;      // TMA descriptors (host copy)
  cudaGraphExec_t graph2[2] = {nullptr, nullptr};   // two-step graphs by starting parity
};

static void drop_graphs(ofd_handle *h) {
  for (int p = 0; p < 2; ++p)
    if (h->graph2[p]) {
      cudaGraphExecDestroy(h->graph2[p]);
      h->graph2[p] = nullptr;
    }
}

namespace {

struct Layout {
  Geom g;
  int z0;
  size_t esize;
  long field_elems;   // per field (2 levels), rounded for 256-B alignment
  long media_elems;
};

size_t storage_size(int st) {
  switch (st) {
    case OFD_F32: return 4;
    case OFD_F64: return 8;
    case OFD_F16: case OFD_BF16: return 2;
  }
  return 0;
}

int check_config(const ofd_config *c) {
  if (!c) return fail(OFD_EINVAL, "null config");
  if (c->space_order != 2 && c->space_order != 4 && c->space_order != 6 && c->space_order != 8)
    return fail(OFD_EINVAL, "space_order %d not supported (2, 4, 6, 8)", c->space_order);
  if (storage_size(c->storage) == 0) return fail(OFD_EINVAL, "unknown storage %d", c->storage);
  const int m = c->space_order / 2;
  for (int i = 0; i < 3; ++i) {
    if (c->dim[i] < 4 * m + 2) return fail(OFD_EINVAL, "dim%d = %d too small for space order %d", i + 1, c->dim[i], c->space_order);
    if (c->dim[i] > (1 << 20)) return fail(OFD_EINVAL, "dim%d = %d too large", i + 1, c->dim[i]);
    if (!(c->spacing[i] > 0)) return fail(OFD_EINVAL, "spacing %d must be > 0", i + 1);
  }
  if (!(c->dt > 0)) return fail(OFD_EINVAL, "dt must be > 0");
  for (int i = 0; i < 6; ++i)
    if (c->free_surface[i] < 0 || c->free_surface[i] > 2) return fail(OFD_EINVAL, "bad free_surface[%d]", i);
  if (c->rounding != OFD_ROUND_NEAREST && c->rounding != OFD_ROUND_STOCHASTIC)
    return fail(OFD_EINVAL, "unknown rounding mode %d", c->rounding);
  return OFD_OK;
}

Layout make_layout(const ofd_config *c) {
  Layout L;
  L.esize = storage_size(c->storage);
  const int m = c->space_order / 2;
  const int A = (int)(128 / L.esize);     // elements per 128 B
  // z = m sits 32 bytes into a 128-byte line: the sweeps' tile rows stay on
  // 32-byte sectors (TMA boxes start on 16-byte boundaries), and the lower
  // z-face ghosts [m-R, m) share a 64-byte DRAM burst with the interior
  // values [m, m+R) they mirror (measured: z-face ghost phases 16 % faster,
  // sweeps unchanged)
  L.z0 = (A - (m % A)) % A + 32 / (int)L.esize;
  const long P = ((long)(L.z0 + c->dim[2]) + A - 1) / A * A;
  L.g.n1 = c->dim[0];
  L.g.n2 = c->dim[1];
  L.g.n3 = c->dim[2];
  L.g.m = m;
  L.g.P = P;
  L.g.plane = (long)c->dim[1] * P;
  const long lvl = (long)c->dim[0] * L.g.plane;
  // keep every level / field base 256-B aligned
  const long align_e = (long)(256 / L.esize);
  L.g.level = (lvl + align_e - 1) / align_e * align_e;
  L.field_elems = 2 * L.g.level;
  // media are float; their own pitch must match field geometry, so they use
  // the float layout with the same z0 rule
  L.media_elems = 0;
  return L;
}

Geom media_geom(const ofd_config *c, int *z0) {
  ofd_config f = *c;
  f.storage = OFD_F32;
  Layout L = make_layout(&f);
  *z0 = L.z0;
  return L.g;
}

CUtensorMapDataType tma_type(int storage) {
  switch (storage) {
    case OFD_F16: return CU_TENSOR_MAP_DATA_TYPE_FLOAT16;
    case OFD_BF16: return CU_TENSOR_MAP_DATA_TYPE_BFLOAT16;
    case OFD_F64: return CU_TENSOR_MAP_DATA_TYPE_FLOAT64;
  }
  return CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
}

// cuTensorMapEncodeTiled, looked up through the runtime's driver entry
// point so that the library does not link libcuda itself and loads on
// machines without a driver (it fails at ofd_create there instead).
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeTiledFn)p;
  });
  return fn;
}

// 3D descriptor over one level: dims (P, n2, n1), rows of P elements.
bool encode(CUtensorMap *m, void *level_base, CUtensorMapDataType t, size_t es, const Geom &g, int bw, int bh) {
  EncodeTiledFn cuTensorMapEncodeTiled = encode_fn();
  if (!cuTensorMapEncodeTiled) return false;
  cuuint64_t dims[3] = {(cuuint64_t)g.P, (cuuint64_t)g.n2, (cuuint64_t)g.n1};
  cuuint64_t strides[2] = {(cuuint64_t)(g.P * es), (cuuint64_t)(g.plane * es)};
  cuuint32_t box[3] = {(cuuint32_t)bw, (cuuint32_t)bh, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = cuTensorMapEncodeTiled(m, t, 3, level_base, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                      CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                                      CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

// Descriptors for every field level (halo and point boxes) and media array.
// Returns false (tiled path off) if any encoding is rejected.
bool build_maps(ofd_handle *h) {
  TmaMaps *mp = new TmaMaps();
  const Geom &g = h->s.g;
  int hw, hh, pw, ph;
  tiled_boxes(h->s.R, (int)h->s.esize, &hw, &hh, &pw, &ph);
  const CUtensorMapDataType t = tma_type(h->s.storage);
  bool ok = hw <= 256 && hh <= 256;
  for (int f = 0; f < NF && ok; ++f)
    for (int l = 0; l < 2 && ok; ++l) {
      char *base = (char *)h->s.field[f] - (size_t)h->s.z0 * h->s.esize + (size_t)l * g.level * h->s.esize;
      ok = encode(&mp->halo[f][l], base, t, h->s.esize, g, hw, hh) &&
           encode(&mp->point[f][l], base, t, h->s.esize, g, pw, ph);
    }
  for (int i = 0; i < NM && ok; ++i)
    ok = encode(&mp->media[i], (void *)(h->s.media[i] - h->s.z0), CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, g, pw, ph);
  if (ok) {
    int bw, bh;
    beta_box(h->s.R, &bw, &bh);
    ok = encode(&mp->beta, (void *)(h->s.media[M_BETA] - h->s.z0), CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, g, bw, bh);
  }
  if (!ok) {
    delete mp;
    return false;
  }
  mp->ok = 1;
  h->maps = mp;
  return true;
}

}  // namespace

namespace ofd {
// ofd_segy.cu
cudaError_t segy_decode(const void *file, long file_size, int nx, int ny, int nz, int swap, float *out);
}  // namespace ofd

extern "C" {

const char *ofd_last_error(void) { return g_last_error.c_str(); }

int ofd_footprint(const ofd_config *cfg, size_t *bytes) {
  int rc = check_config(cfg);
  if (rc) return rc;
  Layout L = make_layout(cfg);
  int mz0;
  Geom mg = media_geom(cfg, &mz0);
  *bytes = (size_t)L.field_elems * L.esize * NF + (size_t)mg.level * sizeof(float) * NM + 4096;
  if (cfg->space_order == 4) {
    // generated-ghost buffers: twelve recompute planes and the literal table
    const long a = std::max((long)cfg->dim[1] * cfg->dim[2],
                            std::max((long)cfg->dim[0] * cfg->dim[2], (long)cfg->dim[0] * cfg->dim[1]));
    *bytes += sizeof(float) * 12 * (size_t)a + 8192;
  }
  return OFD_OK;
}

int ofd_create(const ofd_config *cfg, ofd_handle **out) {
  if (!out) return fail(OFD_EINVAL, "null out");
  *out = nullptr;
  int rc = check_config(cfg);
  if (rc) return rc;
  ofd_handle *h = new ofd_handle();
  h->cfg = *cfg;
  Layout L = make_layout(cfg);
  int mz0;
  Geom mg = media_geom(cfg, &mz0);
  // Media use the float layout; kernels index media with the field geometry,
  // so the two must coincide element for element.  For 16-bit or 64-bit
  // storage the field layout differs, so media are laid out with the field
  // geometry (pitch/z0) but float elements.
  h->s.g = L.g;
  h->s.z0 = L.z0;
  h->s.storage = cfg->storage;
  h->s.esize = L.esize;
  h->s.R = cfg->space_order / 2;
  (void)mg;
  h->level_elems = L.g.level;
  h->field_bytes = (size_t)L.field_elems * L.esize;
  h->media_elems = L.g.level;  // media share the field geometry
  h->media_bytes = (size_t)h->media_elems * sizeof(float);
  cudaGetDevice(&h->device);
  cudaError_t e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) { delete h; return fail(OFD_ECUDA, "cudaStreamCreate: %s", cudaGetErrorString(e)); }
  e = cudaMalloc(&h->fields_raw, h->field_bytes * NF);
  if (e != cudaSuccess) {
    cudaStreamDestroy(h->stream);
    delete h;
    cudaGetLastError();
    return fail(OFD_ENOMEM, "cudaMalloc of %zu field bytes failed: %s", h->field_bytes * NF, cudaGetErrorString(e));
  }
  e = cudaMalloc(&h->media_raw, h->media_bytes * NM + 4 * 4096);
  if (e != cudaSuccess) {
    cudaFree(h->fields_raw);
    cudaStreamDestroy(h->stream);
    delete h;
    cudaGetLastError();
    return fail(OFD_ENOMEM, "cudaMalloc of %zu media bytes failed: %s", h->media_bytes * NM, cudaGetErrorString(e));
  }
  cudaMemsetAsync(h->fields_raw, 0, h->field_bytes * NF, h->stream);
  cudaMemsetAsync(h->media_raw, 0, h->media_bytes * NM + 4 * 4096, h->stream);
  char *fb = (char *)h->fields_raw;
  for (int f = 0; f < NF; ++f) h->s.field[f] = fb + f * h->field_bytes + (size_t)L.z0 * L.esize;
  char *mb = (char *)h->media_raw;
  // media element (x,y,z) at the same linear offset as the field element
  for (int i = 0; i < NM; ++i) h->s.media[i] = (float *)(mb + i * h->media_bytes) + L.z0;
  char *extra = mb + NM * h->media_bytes;
  h->s.d_partial = (double *)extra;                    // 2048 doubles = 16 KB? keep 1152 used
  h->s.d_step = (long *)(extra + 2 * 4096 + 1024);
  h->d_out = (double *)(extra + 2 * 4096 + 2048);
  h->d_err = (int *)(extra + 3 * 4096);
  h->s.d_bar = (unsigned *)(extra + 3 * 4096 + 256);
  h->s.persistent = 0;
  h->s.d_wav = nullptr;
  h->s.src_off = -1;
  h->s.nrec = 0;
  h->s.rec_cap = 0;
  h->s.d_rec = nullptr;
  h->s.d_traces = nullptr;
  h->s.nt = 0;
  for (int f = 0; f < NF; ++f) h->s.scale[f] = cfg->field_scale[f] > 0 ? cfg->field_scale[f] : 1.f;
  if (cfg->storage == OFD_F32 || cfg->storage == OFD_F64)
    for (int f = 0; f < NF; ++f) h->s.scale[f] = 1.f;
  for (int i = 0; i < 6; ++i) h->s.face[i] = cfg->free_surface[i];
  h->s.legacy = cfg->legacy_bc;
  h->s.sr = cfg->rounding == OFD_ROUND_STOCHASTIC ? 1 : 0;
  h->s.gen_ghost = 0;
  h->s.d_kg = nullptr;
  h->s.d_rc = nullptr;
  h->s.rcs = 0;
  h->s.st2 = nullptr;
  h->s.ev_fork = h->s.ev_join = nullptr;
  h->s.rc_mode = OFD_RC_MODE_DEFAULT;
  h->s.rc_bps = OFD_RC_BPS_DEFAULT;
  h->s.dt = cfg->dt;
  for (int i = 0; i < 3; ++i) h->s.h[i] = cfg->spacing[i];
  for (int k = 0; k < 4; ++k) h->s.c[k] = cfg->weights[k];
  h->s.variant = cfg->kernel_variant;
  h->s.var_stress = 0;
  h->s.var_velocity = 0;
  h->s.chunk_waves = 1;
  h->s.plain_bx = 32;
  h->s.plain_by = 8;
  h->s.het = 0;
  h->s.nks = h->s.nkv = 0;
  switch (cfg->storage) {
    case OFD_F32: h->be = backend_for<float>(h->s.R); break;
    case OFD_F64: h->be = backend_for<double>(h->s.R); break;
    case OFD_F16: h->be = backend_for<__half>(h->s.R); break;
    case OFD_BF16: h->be = backend_for<__nv_bfloat16>(h->s.R); break;
  }
  h->s.tiled.maps = nullptr;
  h->s.tiled.err = h->d_err;
  h->s.tiled.z0 = L.z0;
  h->s.tiled.waves = 1;
  h->s.tiled.kd[0] = h->s.tiled.kd[1] = 0;
  h->s.tiled.wait_ns = 10000000000ULL;
  if (!encode_fn()) {
    ofd_destroy(h);
    return fail(OFD_ECUDA, "the driver does not provide cuTensorMapEncodeTiled");
  }
  if (build_maps(h)) h->s.tiled.maps = h->maps;
  e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess || !h->be) {
    int code = fail(OFD_ECUDA, "initialisation failed: %s", cudaGetErrorString(e));
    ofd_destroy(h);
    return code;
  }
  *out = h;
  return OFD_OK;
}

int ofd_destroy(ofd_handle *h) {
  if (!h) return OFD_OK;
  if (h->stream) cudaStreamSynchronize(h->stream);
  drop_graphs(h);
  delete h->be;
  delete h->maps;
  if (h->s.d_wav) cudaFree(h->s.d_wav);
  if (h->s.d_kg) cudaFree(h->s.d_kg);
  if (h->s.d_rc) cudaFree(h->s.d_rc);
  if (h->s.st2) {
    cudaStreamSynchronize(h->s.st2);
    cudaStreamDestroy(h->s.st2);
  }
  if (h->s.ev_fork) cudaEventDestroy(h->s.ev_fork);
  if (h->s.ev_join) cudaEventDestroy(h->s.ev_join);
  if (h->s.d_rec) cudaFree(h->s.d_rec);
  if (h->s.d_traces) cudaFree(h->s.d_traces);
  if (h->fields_raw) cudaFree(h->fields_raw);
  if (h->media_raw) cudaFree(h->media_raw);
  if (h->stream) cudaStreamDestroy(h->stream);
  if (h->copy_stream) cudaStreamDestroy(h->copy_stream);
  delete h;
  return OFD_OK;
}

void *ofd_stream(ofd_handle *h) { return h ? (void *)h->stream : nullptr; }

int ofd_set_coefficients(ofd_handle *h, int het, const float *ks, int nks, const float *kv, int nkv) {
  if (!h || !ks || !kv) return fail(OFD_EINVAL, "null argument");
  if (het != 0 && het != 1) return fail(OFD_EINVAL, "het must be 0 or 1");
  const int es = h->be->table_size(het, 1), ev = h->be->table_size(het, 0);
  if (nks != es || nkv != ev)
    return fail(OFD_EINVAL, "coefficient tables of size %d/%d do not match the prebuilt %s expression of space order %d (%d/%d)",
                nks, nkv, het ? "heterogeneous" : "constant-media", h->cfg.space_order, es, ev);
  h->s.het = het;
  h->s.nks = nks;
  h->s.nkv = nkv;
  for (int i = 0; i < nks; ++i) h->s.Ks[i] = ks[i];
  for (int i = 0; i < nkv; ++i) h->s.Kv[i] = kv[i];
  h->s.tiled.kd[1] = het && h->be->kmap_ok(h->s, true) ? 1 : 0;
  h->s.tiled.kd[0] = het && h->be->kmap_ok(h->s, false) ? 1 : 0;
  h->be->prepare(h->s);
  drop_graphs(h);
  OFD_CUDA(cudaGetLastError());
  return OFD_OK;
}

int ofd_set_ghost_coefficients(ofd_handle *h, int het, const float *kg, int nkg) {
  if (!h) return fail(OFD_EINVAL, "null handle");
  if (nkg == 0) {
    h->s.gen_ghost = 0;
    drop_graphs(h);
    return OFD_OK;
  }
  if (!kg) return fail(OFD_EINVAL, "null table");
  if (het != 0 && het != 1) return fail(OFD_EINVAL, "het must be 0 or 1");
  if (h->s.nks == 0 || het != h->s.het)
    return fail(OFD_ESTATE, "set the update coefficients of the same media mode first");
  const int want = h->be->ghost_table_size(het);
  if (want == 0)
    return fail(OFD_EINVAL, "no generated ghost expressions for space order %d and this storage", h->cfg.space_order);
  if (nkg != want)
    return fail(OFD_EINVAL, "ghost coefficient table of size %d does not match the prebuilt expressions (%d)", nkg, want);
  for (int i = 0; i < 6; ++i)
    if (h->cfg.free_surface[i] != OFD_BC_LEVANDER)
      return fail(OFD_EINVAL, "generated ghost expressions need Levander free surfaces on all six faces");
  OFD_CUDA(cudaStreamSynchronize(h->stream));
  if (!h->s.d_kg) OFD_CUDA(cudaMalloc((void **)&h->s.d_kg, sizeof(float) * (size_t)want));
  if (!h->s.d_rc) {
    // recompute values of one step (12 face planes), computed on a second
    // stream while the stress sweep runs
    const Geom &g = h->s.g;
    const long rcs = std::max((long)g.n2 * g.n3, std::max((long)g.n1 * g.n3, (long)g.n1 * g.n2));
    OFD_CUDA(cudaMalloc((void **)&h->s.d_rc, sizeof(float) * 12 * (size_t)rcs));
    h->s.rcs = rcs;
    OFD_CUDA(cudaStreamCreateWithPriority(&h->s.st2, cudaStreamNonBlocking, greatest_priority()));
    OFD_CUDA(cudaEventCreateWithFlags(&h->s.ev_fork, cudaEventDisableTiming));
    OFD_CUDA(cudaEventCreateWithFlags(&h->s.ev_join, cudaEventDisableTiming));
  }
  OFD_CUDA(cudaMemcpyAsync(h->s.d_kg, kg, sizeof(float) * (size_t)nkg, cudaMemcpyHostToDevice, h->stream));
  OFD_CUDA(cudaStreamSynchronize(h->stream));
  h->s.gen_ghost = 1;
  drop_graphs(h);
  return OFD_OK;
}

int ofd_set_media_const(ofd_handle *h, float beta, float lambda, float mu) {
  if (!h) return fail(OFD_EINVAL, "null handle");
  const long n = h->media_elems;
  const float vals[NM] = {lambda, mu, mu, mu, mu, beta, beta, beta, beta};
  for (int i = 0; i < NM; ++i)
    fill_kernel<<<1216, 256, 0, h->stream>>>(h->s.media[i] - h->s.z0, n, vals[i]);
  OFD_CUDA(cudaGetLastError());
  OFD_CUDA(cudaStreamSynchronize(h->stream));
  return OFD_OK;
}

// Queue the media preprocessing on the handle's stream: rho, vp, vs (host or
// device memory, dense reference layout) in, the nine effective-media arrays
// out.  The three inputs and 1/mu pass through one stream-ordered scratch
// allocation.  The inputs move in x slabs on the handle's copy stream, and
// each slab's per-point kernel starts as soon as its copies land (an event),
// so the upload overlaps the FP64 preprocessing; a slab's averaging kernel,
// which reads the next plane, follows the next slab's per-point kernel.
static int queue_media(ofd_handle *h, const float *rho, const float *vp, const float *vs, cudaMemcpyKind kind) {
  const Geom &g = h->s.g;
  const long n = (long)g.n1 * g.n2 * g.n3;
  const long plane = (long)g.n2 * g.n3;
  float *tmp = nullptr;
  // three float inputs, then 1/mu in double (8-byte aligned: 3n floats = 12n bytes)
  OFD_CUDA(scratch_alloc((void **)&tmp, sizeof(float) * n * 3 + sizeof(double) * n + 16, h->stream));
  double *inv_mu = (double *)(((uintptr_t)(tmp + 3 * n) + 15) & ~(uintptr_t)15);
  if (!h->copy_stream) OFD_CUDA(cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking));
  auto order = [](cudaStream_t from, cudaStream_t to) -> cudaError_t {
    cudaEvent_t ev;
    cudaError_t e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventRecord(ev, from);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(to, ev, 0);
    cudaEventDestroy(ev);   // released once it has completed
    return e;
  };
  OFD_CUDA(order(h->stream, h->copy_stream));   // the scratch exists before the copies
  const dim3 blk(32, 8);
  const int nslab = g.n1 < 8 ? g.n1 : 8;
  int px0 = -1, px1 = -1;
  auto avg = [&](int x0, int x1) {
    const dim3 grd((g.n3 + 31) / 32, (g.n2 + 7) / 8, x1 - x0);
    media_avg_kernel<<<grd, blk, 0, h->stream>>>(h->s.media[M_BETA], inv_mu, g, h->s.media[M_MU12],
                                                 h->s.media[M_MU13], h->s.media[M_MU23], h->s.media[M_B1],
                                                 h->s.media[M_B2], h->s.media[M_B3], x0);
  };
  for (int k = 0; k < nslab; ++k) {
    const int x0 = (int)((long)g.n1 * k / nslab), x1 = (int)((long)g.n1 * (k + 1) / nslab);
    const long off = (long)x0 * plane, cnt = (long)(x1 - x0) * plane;
    OFD_CUDA(cudaMemcpyAsync(tmp + off, rho + off, sizeof(float) * cnt, kind, h->copy_stream));
    OFD_CUDA(cudaMemcpyAsync(tmp + n + off, vp + off, sizeof(float) * cnt, kind, h->copy_stream));
    OFD_CUDA(cudaMemcpyAsync(tmp + 2 * n + off, vs + off, sizeof(float) * cnt, kind, h->copy_stream));
    OFD_CUDA(order(h->copy_stream, h->stream));
    const dim3 grd((g.n3 + 31) / 32, (g.n2 + 7) / 8, x1 - x0);
    media_point_kernel<<<grd, blk, 0, h->stream>>>(tmp, tmp + n, tmp + 2 * n, g, h->s.media[M_BETA],
                                                   h->s.media[M_LAM], h->s.media[M_MU], inv_mu, x0);
    if (px0 >= 0) avg(px0, px1);   // its x + 1 plane (x0) is done now
    px0 = x0;
    px1 = x1;
  }
  avg(px0, px1);
  OFD_CUDA(cudaGetLastError());
  OFD_CUDA(cudaFreeAsync(tmp, h->stream));
  return OFD_OK;
}

int ofd_set_media(ofd_handle *h, const float *rho, const float *vp, const float *vs) {
  if (!h || !rho || !vp || !vs) return fail(OFD_EINVAL, "null argument");
  const int rc = queue_media(h, rho, vp, vs, cudaMemcpyDefault);
  if (rc) return rc;
  OFD_CUDA(cudaStreamSynchronize(h->stream));
  return OFD_OK;
}

int ofd_set_media_async(ofd_handle *h, const float *rho, const float *vp, const float *vs) {
  if (!h || !rho || !vp || !vs) return fail(OFD_EINVAL, "null argument");
  return queue_media(h, rho, vp, vs, cudaMemcpyDefault);
}

static int check_fl(ofd_handle *h, int field, int level) {
  if (!h) return fail(OFD_EINVAL, "null handle");
  if (field < 0 || field >= NF) return fail(OFD_EINVAL, "bad field %d", field);
  if (level < 0 || level > 1) return fail(OFD_EINVAL, "bad level %d", level);
  return OFD_OK;
}

int ofd_upload_field_device(ofd_handle *h, int field, int level, const float *dev) {
  int rc = check_fl(h, field, level);
  if (rc) return rc;
  h->be->to_padded(h->s, dev, field, level, h->stream);
  OFD_CUDA(cudaGetLastError());
  return OFD_OK;
}

int ofd_download_field_device(ofd_handle *h, int field, int level, float *dev) {
  int rc = check_fl(h, field, level);
  if (rc) return rc;
  h->be->from_padded(h->s, dev, field, level, h->stream);
  OFD_CUDA(cudaGetLastError());
  return OFD_OK;
}

// Host <-> device field transfers in stream order.  FP32 storage copies the
// padded rows straight to/from the dense host array (one pitched copy: rows of
// dim3 floats at the padded pitch); other storage types convert through a
// stream-ordered dense FP32 scratch array.
static int queue_upload(ofd_handle *h, int field, int level, const float *host) {
  const Geom &g = h->s.g;
  if (h->s.storage == OFD_F32) {
    float *dst = (float *)h->s.field[field] + (size_t)level * g.level;
    OFD_CUDA(cudaMemcpy2DAsync(dst, sizeof(float) * g.P, host, sizeof(float) * g.n3, sizeof(float) * g.n3,
                               (size_t)g.n1 * g.n2, cudaMemcpyDefault, h->stream));
    return OFD_OK;
  }
  const long n = (long)g.n1 * g.n2 * g.n3;
  float *tmp = nullptr;
  OFD_CUDA(scratch_alloc((void **)&tmp, sizeof(float) * n, h->stream));
  OFD_CUDA(cudaMemcpyAsync(tmp, host, sizeof(float) * n, cudaMemcpyDefault, h->stream));
  h->be->to_padded(h->s, tmp, field, level, h->stream);
  OFD_CUDA(cudaGetLastError());
  OFD_CUDA(cudaFreeAsync(tmp, h->stream));
  return OFD_OK;
}

static int queue_download(ofd_handle *h, int field, int level, float *host) {
  const Geom &g = h->s.g;
  if (h->s.storage == OFD_F32) {
    const float *src = (const float *)h->s.field[field] + (size_t)level * g.level;
    OFD_CUDA(cudaMemcpy2DAsync(host, sizeof(float) * g.n3, src, sizeof(float) * g.P, sizeof(float) * g.n3,
                               (size_t)g.n1 * g.n2, cudaMemcpyDefault, h->stream));
    return OFD_OK;
  }
  const long n = (long)g.n1 * g.n2 * g.n3;
  float *tmp = nullptr;
  OFD_CUDA(scratch_alloc((void **)&tmp, sizeof(float) * n, h->stream));
  h->be->from_padded(h->s, tmp, field, level, h->stream);
  OFD_CUDA(cudaGetLastError());
  OFD_CUDA(cudaMemcpyAsync(host, tmp, sizeof(float) * n, cudaMemcpyDefault, h->stream));
  OFD_CUDA(cudaFreeAsync(tmp, h->stream));
  return OFD_OK;
}

int ofd_upload_field(ofd_handle *h, int field, int level, const float *host) {
  int rc = check_fl(h, field, level);
  if (rc) return rc;
  if (!host) return fail(OFD_EINVAL, "null host array");
  rc = queue_upload(h, field, level, host);
  if (rc) return rc;
  OFD_CUDA(cudaStreamSynchronize(h->stream));
  return OFD_OK;
}

int ofd_download_field(ofd_handle *h, int field, int level, float *host) {
  int rc = check_fl(h, field, level);
  if (rc) return rc;
  if (!host) return fail(OFD_EINVAL, "null host array");
  rc = queue_download(h, field, level, host);
  if (rc) return rc;
  OFD_CUDA(cudaStreamSynchronize(h->stream));
  return OFD_OK;
}

int ofd_upload_field_async(ofd_handle *h, int field, int level, const float *host) {
  int rc = check_fl(h, field, level);
  if (rc) return rc;
  if (!host) return fail(OFD_EINVAL, "null host array");
  return queue_upload(h, field, level, host);
}

int ofd_download_field_async(ofd_handle *h, int field, int level, float *host) {
  int rc = check_fl(h, field, level);
  if (rc) return rc;
  if (!host) return fail(OFD_EINVAL, "null host array");
  return queue_download(h, field, level, host);
}

// FP64 storage: double host arrays copied as they are, one pitched copy.
static int transfer_f64(ofd_handle *h, int field, int level, double *host, bool up) {
  int rc = check_fl(h, field, level);
  if (rc) return rc;
  if (!host) return fail(OFD_EINVAL, "null host array");
  if (h->s.storage != OFD_F64) return fail(OFD_EINVAL, "FP64 field transfers need OFD_F64 storage");
  const Geom &g = h->s.g;
  double *dev = (double *)h->s.field[field] + (size_t)level * g.level;
  const size_t row = sizeof(double) * g.n3, pitch = sizeof(double) * g.P, rows = (size_t)g.n1 * g.n2;
  if (up)
    OFD_CUDA(cudaMemcpy2DAsync(dev, pitch, host, row, row, rows, cudaMemcpyDefault, h->stream));
  else
    OFD_CUDA(cudaMemcpy2DAsync(host, row, dev, pitch, row, rows, cudaMemcpyDefault, h->stream));
  OFD_CUDA(cudaStreamSynchronize(h->stream));
  return OFD_OK;
}

int ofd_upload_field_f64(ofd_handle *h, int field, int level, const double *host) {
  return transfer_f64(h, field, level, const_cast<double *>(host), true);
}

int ofd_download_field_f64(ofd_handle *h, int field, int level, double *host) {
  return transfer_f64(h, field, level, host, false);
}

int ofd_zero_fields(ofd_handle *h) {
  if (!h) return fail(OFD_EINVAL, "null handle");
  OFD_CUDA(cudaMemsetAsync(h->fields_raw, 0, h->field_bytes * NF, h->stream));
  return OFD_OK;
}

int ofd_set_source_xyz(ofd_handle *h, int sx, int sy, int sz, const float *wx, const float *wy, const float *wz,
                       int nt) {
  if (!h) return fail(OFD_EINVAL, "null handle");
  const Geom &g = h->s.g;
  if (nt <= 0 || !wx || !wy || !wz) {
    h->s.src_off = -1;
    return OFD_OK;
  }
  if (sx < 0 || sx >= g.n1 || sy < 0 || sy >= g.n2 || sz < 0 || sz >= g.n3)
    return fail(OFD_EINVAL, "source (%d,%d,%d) outside the grid", sx, sy, sz);
  if (h->s.d_wav) {
    OFD_CUDA(cudaStreamSynchronize(h->stream));
    cudaFree(h->s.d_wav);
    h->s.d_wav = nullptr;
  }
  // the x, y and z signals back to back, nt values each
  OFD_CUDA(cudaMalloc((void **)&h->s.d_wav, sizeof(float) * 3 * (size_t)nt));
  // stream-ordered copies: a plain cudaMemcpy from pageable memory may return
  // before its DMA lands and is not ordered with this non-blocking stream
  const float *w[3] = {wx, wy, wz};
  for (int q = 0; q < 3; ++q)
    OFD_CUDA(cudaMemcpyAsync(h->s.d_wav + (size_t)q * nt, w[q], sizeof(float) * nt, cudaMemcpyHostToDevice,
                             h->stream));
  OFD_CUDA(cudaStreamSynchronize(h->stream));
  h->s.nt = nt;
  h->s.src_off = (long)sx * g.plane + (long)sy * g.P + sz;
  drop_graphs(h);
  return OFD_OK;
}

int ofd_set_source(ofd_handle *h, int sx, int sy, int sz, const float *wavelet, int nt) {
  return ofd_set_source_xyz(h, sx, sy, sz, wavelet, wavelet, wavelet, nt);
}

int ofd_set_receivers(ofd_handle *h, int nrec, const int *ijk, int nt_cap) {
  if (!h) return fail(OFD_EINVAL, "null handle");
  if (nrec < 0 || nt_cap < 0 || (nrec > 0 && (!ijk || nt_cap == 0)))
    return fail(OFD_EINVAL, "bad receiver arguments");
  const Geom &g = h->s.g;
  std::vector<long> off(nrec);
  for (int i = 0; i < nrec; ++i) {
    const int x = ijk[3 * i], y = ijk[3 * i + 1], z = ijk[3 * i + 2];
    if (x < 0 || x >= g.n1 || y < 0 || y >= g.n2 || z < 0 || z >= g.n3)
      return fail(OFD_EINVAL, "receiver %d at (%d,%d,%d) outside the grid", i, x, y, z);
    off[i] = (long)x * g.plane + (long)y * g.P + z;
  }
  if ((double)nt_cap * 4.0 * nrec * sizeof(float) > 64e9)
    return fail(OFD_EINVAL, "trace buffer of %d steps x %d receivers is too large", nt_cap, nrec);
  OFD_CUDA(cudaStreamSynchronize(h->stream));
  if (h->s.d_rec) cudaFree(h->s.d_rec);
  if (h->s.d_traces) cudaFree(h->s.d_traces);
  h->s.d_rec = nullptr;
  h->s.d_traces = nullptr;
  h->s.nrec = 0;
  h->s.rec_cap = 0;
  drop_graphs(h);
  if (nrec == 0) return OFD_OK;
  const size_t tbytes = sizeof(float) * 4 * (size_t)nrec * nt_cap;
  if (cudaMalloc((void **)&h->s.d_rec, sizeof(long) * nrec) != cudaSuccess ||
      cudaMalloc((void **)&h->s.d_traces, tbytes) != cudaSuccess) {
    cudaGetLastError();
    return fail(OFD_ENOMEM, "cannot allocate %zu bytes of traces", tbytes);
  }
  OFD_CUDA(cudaMemcpyAsync(h->s.d_rec, off.data(), sizeof(long) * nrec, cudaMemcpyHostToDevice, h->stream));
  OFD_CUDA(cudaMemsetAsync(h->s.d_traces, 0, tbytes, h->stream));
  OFD_CUDA(cudaStreamSynchronize(h->stream));
  h->s.nrec = nrec;
  h->s.rec_cap = nt_cap;
  return OFD_OK;
}

int ofd_get_traces(ofd_handle *h, float *host) {
  if (!h || !host) return fail(OFD_EINVAL, "null argument");
  if (h->s.nrec == 0) return fail(OFD_ESTATE, "no receivers set");
  const size_t tbytes = sizeof(float) * 4 * (size_t)h->s.nrec * h->s.rec_cap;
  OFD_CUDA(cudaMemcpyAsync(host, h->s.d_traces, tbytes, cudaMemcpyDeviceToHost, h->stream));
  OFD_CUDA(cudaStreamSynchronize(h->stream));
  return OFD_OK;
}

int ofd_apply_boundary_init(ofd_handle *h, int level) {
  if (!h) return fail(OFD_EINVAL, "null handle");
  if (level < 0 || level > 1) return fail(OFD_EINVAL, "bad level %d", level);
  h->be->boundary_init(h->s, level, h->stream);
  OFD_CUDA(cudaGetLastError());
  return OFD_OK;
}

int ofd_set_step(ofd_handle *h, long steps) {
  if (!h || steps < 0) return fail(OFD_EINVAL, "bad argument");
  h->steps = steps;
  OFD_CUDA(cudaMemcpyAsync(h->s.d_step, &h->steps, sizeof(long), cudaMemcpyHostToDevice, h->stream));
  OFD_CUDA(cudaStreamSynchronize(h->stream));
  return OFD_OK;
}

int ofd_get_step(ofd_handle *h, long *steps) {
  if (!h || !steps) return fail(OFD_EINVAL, "bad argument");
  *steps = h->steps;
  return OFD_OK;
}

// nsteps in cooperative launches of at most 1024 steps each
static int run_persistent(ofd_handle *h, int nsteps) {
  int done = 0;
  while (done < nsteps) {
    const int k = nsteps - done < 1024 ? nsteps - done : 1024;
    const int e = h->be->step_persistent(h->s, (int)(h->steps & 1), k, h->stream);
    if (e != (int)cudaSuccess)
      return fail(OFD_ECUDA, "persistent launch failed: %s", cudaGetErrorString((cudaError_t)e));
    h->steps += k;
    done += k;
  }
  return OFD_OK;
}

int ofd_set_persistent(ofd_handle *h, int enable) {
  if (!h) return fail(OFD_EINVAL, "null handle");
  int dev = 0, coop = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
  if (enable && !coop) return fail(OFD_EINVAL, "device has no cooperative launch");
  h->s.persistent = enable ? 1 : 0;
  return OFD_OK;
}

int ofd_step(ofd_handle *h, int nsteps) {
  if (!h) return fail(OFD_EINVAL, "null handle");
  if (nsteps < 0) return fail(OFD_EINVAL, "nsteps < 0");
  if (h->s.nks == 0) return fail(OFD_ESTATE, "ofd_set_coefficients has not been called");
  if (h->s.persistent) return run_persistent(h, nsteps);
  for (int i = 0; i < nsteps; ++i) {
    const int t0 = (int)(h->steps & 1);
    h->be->step(h->s, t0, h->stream);
    h->steps += 1;
  }
  OFD_CUDA(cudaGetLastError());
  return OFD_OK;
}

static int check_err_word(ofd_handle *h) {
  int err = 0;
  OFD_CUDA(cudaMemcpyAsync(&err, h->d_err, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  OFD_CUDA(cudaStreamSynchronize(h->stream));
  if (err) {
    cudaMemsetAsync(h->d_err, 0, sizeof(int), h->stream);
    cudaStreamSynchronize(h->stream);
    return fail(OFD_ETIMEOUT, "a bounded device wait expired (error word %d: %s)", err,
                err == 3 ? "grid barrier of the persistent kernel" : "pipeline wait of a tiled sweep");
  }
  return OFD_OK;
}

int ofd_step_profiled(ofd_handle *h, int nsteps, double *ms_total, double ms_class[4], long *launches) {
  if (!h || !ms_total || !ms_class) return fail(OFD_EINVAL, "null argument");
  if (nsteps <= 0) return fail(OFD_EINVAL, "nsteps must be > 0");
  if (h->s.nks == 0) return fail(OFD_ESTATE, "ofd_set_coefficients has not been called");
  std::vector<StepEvents> evs(nsteps);
  for (int i = 0; i < nsteps; ++i)
    for (int k = 0; k < 8; ++k) OFD_CUDA(cudaEventCreate(&evs[i].ev[k]));
  for (int i = 0; i < nsteps; ++i) {
    const int t0 = (int)(h->steps & 1);
    h->be->step(h->s, t0, h->stream, &evs[i]);
    h->steps += 1;
  }
  OFD_CUDA(cudaGetLastError());
  OFD_CUDA(cudaStreamSynchronize(h->stream));
  for (int k = 0; k < 4; ++k) ms_class[k] = 0;
  for (int i = 0; i < nsteps; ++i)
    for (int k = 0; k < 4; ++k) {
      float ms = 0;
      OFD_CUDA(cudaEventElapsedTime(&ms, evs[i].ev[2 * k], evs[i].ev[2 * k + 1]));
      ms_class[k] += ms;
    }
  float tot = 0;
  OFD_CUDA(cudaEventElapsedTime(&tot, evs[0].ev[0], evs[nsteps - 1].ev[7]));
  *ms_total = tot;
  if (launches) *launches = (long)nsteps * h->be->launches_per_step(h->s);
  for (int i = 0; i < nsteps; ++i)
    for (int k = 0; k < 8; ++k) cudaEventDestroy(evs[i].ev[k]);
  return check_err_word(h);
}

int ofd_set_tuning(ofd_handle *h, int stress_variant, int velocity_variant, int chunk_waves, int plain_bx,
                   int plain_by) {
  if (!h) return fail(OFD_EINVAL, "null handle");
  if (stress_variant < 0 || stress_variant > 1 || velocity_variant < 0 || velocity_variant > 1)
    return fail(OFD_EINVAL, "variants are 0 (tiled) or 1 (plain)");
  if (chunk_waves < 1 || chunk_waves > 64) return fail(OFD_EINVAL, "chunk_waves must be in [1, 64]");
  if (plain_bx < 1 || plain_by < 1 || plain_bx * plain_by > 256 || plain_bx % 32)
    return fail(OFD_EINVAL, "plain block must be a multiple of 32 wide and at most 256 threads");
  h->s.var_stress = stress_variant;
  h->s.var_velocity = velocity_variant;
  h->s.chunk_waves = chunk_waves;
  h->s.tiled.waves = chunk_waves;
  h->s.plain_bx = plain_bx;
  h->s.plain_by = plain_by;
  drop_graphs(h);
  return OFD_OK;
}

int ofd_set_wait_limit(ofd_handle *h, double seconds) {
  if (!h) return fail(OFD_EINVAL, "null handle");
  if (!(seconds > 0) || seconds > 600) return fail(OFD_EINVAL, "wait limit must be in (0, 600] seconds");
  h->s.tiled.wait_ns = (unsigned long long)(seconds * 1e9);
  if (h->s.tiled.wait_ns == 0) h->s.tiled.wait_ns = 1;
  drop_graphs(h);
  return OFD_OK;
}

int ofd_set_ghost_schedule(ofd_handle *h, int mode, int blocks_per_sm) {
  if (!h) return fail(OFD_EINVAL, "null handle");
  if (mode != 0 && mode != 1) return fail(OFD_EINVAL, "ghost schedule mode must be 0 (after the sweep) or 1 (beside it)");
  if (blocks_per_sm < 1 || blocks_per_sm > 16) return fail(OFD_EINVAL, "blocks_per_sm must be in [1, 16]");
  h->s.rc_mode = mode;
  h->s.rc_bps = blocks_per_sm;
  drop_graphs(h);
  return OFD_OK;
}

int ofd_step_graph(ofd_handle *h, int nsteps) {
  if (!h) return fail(OFD_EINVAL, "null handle");
  if (nsteps < 0) return fail(OFD_EINVAL, "nsteps < 0");
  if (h->s.nks == 0) return fail(OFD_ESTATE, "ofd_set_coefficients has not been called");
  if (h->s.persistent) return run_persistent(h, nsteps);
  int done = 0;
  while (nsteps - done >= 2) {
    const int p = (int)(h->steps & 1);
    if (!h->graph2[p]) {
      cudaGraph_t g = nullptr;
      OFD_CUDA(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
      h->be->step(h->s, p, h->stream);
      h->be->step(h->s, 1 - p, h->stream);
      cudaError_t e = cudaStreamEndCapture(h->stream, &g);
      if (e != cudaSuccess) return fail(OFD_ECUDA, "graph capture failed: %s", cudaGetErrorString(e));
      e = cudaGraphInstantiate(&h->graph2[p], g, 0);
      cudaGraphDestroy(g);
      if (e != cudaSuccess) return fail(OFD_ECUDA, "graph instantiation failed: %s", cudaGetErrorString(e));
    }
    OFD_CUDA(cudaGraphLaunch(h->graph2[p], h->stream));
    h->steps += 2;
    done += 2;
  }
  if (done < nsteps) {
    h->be->step(h->s, (int)(h->steps & 1), h->stream);
    h->steps += 1;
  }
  OFD_CUDA(cudaGetLastError());
  return OFD_OK;
}

int ofd_step_timed(ofd_handle *h, int nsteps, double *ms, long *launches) {
  if (!h || !ms) return fail(OFD_EINVAL, "null argument");
  if (nsteps <= 0) return fail(OFD_EINVAL, "nsteps must be > 0");
  if (h->s.nks == 0) return fail(OFD_ESTATE, "ofd_set_coefficients has not been called");
  if (h->s.persistent) return fail(OFD_ESTATE, "timed stepping runs the launch path; persistent stepping is on");
  cudaEvent_t a = nullptr, b = nullptr;
  cudaError_t e = cudaEventCreate(&a);
  if (e == cudaSuccess) e = cudaEventCreate(&b);
  if (e == cudaSuccess) e = cudaEventRecord(a, h->stream);
  int rc = OFD_OK;
  if (e == cudaSuccess) {
    rc = ofd_step(h, nsteps);
    if (rc == OFD_OK) e = cudaEventRecord(b, h->stream);
  }
  float f = 0.f;
  if (e == cudaSuccess && rc == OFD_OK) e = cudaEventSynchronize(b);
  if (e == cudaSuccess && rc == OFD_OK) e = cudaEventElapsedTime(&f, a, b);
  if (a) cudaEventDestroy(a);
  if (b) cudaEventDestroy(b);
  if (rc != OFD_OK) return rc;
  if (e != cudaSuccess) return fail(OFD_ECUDA, "event timing: %s", cudaGetErrorString(e));
  *ms = f;
  if (launches) *launches = (long)nsteps * h->be->launches_per_step(h->s);
  return check_err_word(h);
}


// ------------------------------------------------------------- groups

struct ofd_group {
  std::vector<ofd_handle *> members;
  GroupPlanBase *plan = nullptr;
  Backend *be = nullptr;            // members[0]'s backend (same R and storage for all)
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;       // group work finished (member streams wait on it)
  std::vector<cudaEvent_t> ready;   // member work finished (the group waits on it)
  cudaGraphExec_t graph2[2] = {nullptr, nullptr};
  long steps = 0;                   // members' common step count parity source
};

int ofd_group_destroy(ofd_group *g) {
  if (!g) return OFD_OK;
  if (g->stream) cudaStreamSynchronize(g->stream);
  for (int p = 0; p < 2; ++p)
    if (g->graph2[p]) cudaGraphExecDestroy(g->graph2[p]);
  delete g->plan;
  for (cudaEvent_t e : g->ready) cudaEventDestroy(e);
  if (g->done) cudaEventDestroy(g->done);
  if (g->stream) cudaStreamDestroy(g->stream);
  delete g;
  return OFD_OK;
}

int ofd_group_create(ofd_handle *const *hs, int n, int chunk_planes, ofd_group **out) {
  if (!hs || !out || n <= 0) return fail(OFD_EINVAL, "null argument or empty group");
  *out = nullptr;
  ofd_handle *h0 = hs[0];
  if (!h0) return fail(OFD_EINVAL, "null member 0");
  for (int i = 0; i < n; ++i) {
    ofd_handle *h = hs[i];
    if (!h) return fail(OFD_EINVAL, "null member %d", i);
    if (h->device != h0->device) return fail(OFD_EINVAL, "member %d is on another device", i);
    if (h->s.R != h0->s.R || h->s.storage != h0->s.storage)
      return fail(OFD_EINVAL, "member %d has another space order or storage than member 0", i);
    if (h->s.nks == 0) return fail(OFD_ESTATE, "member %d: ofd_set_coefficients has not been called", i);
    if (h->s.het != h0->s.het) return fail(OFD_EINVAL, "member %d has another media mode than member 0", i);
    if ((h->steps & 1) != (h0->steps & 1)) return fail(OFD_EINVAL, "member %d is at another time level", i);
    if (!h->be->tiled_ok(h->s)) return fail(OFD_EINVAL, "member %d cannot use the tiled sweeps (grid too small)", i);
    for (int j = 0; j < i; ++j)
      if (hs[j] == h) return fail(OFD_EINVAL, "member %d appears twice", i);
  }
  ofd_group *g = new ofd_group();
  g->members.assign(hs, hs + n);
  g->be = h0->be;
  g->steps = h0->steps;
  cudaError_t e = cudaSetDevice(h0->device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&g->done, cudaEventDisableTiming);
  g->ready.resize(n, nullptr);
  for (int i = 0; i < n && e == cudaSuccess; ++i) e = cudaEventCreateWithFlags(&g->ready[i], cudaEventDisableTiming);
  if (e == cudaSuccess) {
    std::vector<const DevState *> ms(n);
    for (int i = 0; i < n; ++i) ms[i] = &hs[i]->s;
    g->plan = g->be->group_build(ms.data(), n, chunk_planes, g->stream, &e);
  }
  if (e != cudaSuccess || !g->plan) {
    ofd_group_destroy(g);
    return fail(OFD_ECUDA, "group setup failed: %s", cudaGetErrorString(e));
  }
  *out = g;
  return OFD_OK;
}

int ofd_set_device(int device) {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess) return fail(OFD_ECUDA, "cudaGetDeviceCount: %s", cudaGetErrorString(e));
  if (device < 0 || device >= n) return fail(OFD_EINVAL, "device %d outside 0..%d", device, n - 1);
  e = cudaSetDevice(device);
  if (e != cudaSuccess) return fail(OFD_ECUDA, "cudaSetDevice(%d): %s", device, cudaGetErrorString(e));
  return OFD_OK;
}

int ofd_segy_decode_ibm(const void *file, long file_size, int nx, int ny, int nz, int swap_endian, float *out) {
  if (!file || !out) return fail(OFD_EINVAL, "null argument");
  if (nx <= 0 || ny <= 0 || nz <= 0) return fail(OFD_EINVAL, "bad model dimensions %d x %d x %d", nx, ny, nz);
  const long need = 3600 + (long)nx * ny * (240 + 4L * nz);
  if (file_size < need)
    return fail(OFD_EINVAL, "SEG-Y image of %ld bytes is shorter than its %d x %d traces (%ld bytes)", file_size, nx,
                ny, need);
  const cudaError_t e = ofd::segy_decode(file, file_size, nx, ny, nz, swap_endian, out);
  if (e != cudaSuccess) return fail(OFD_ECUDA, "SEG-Y decode: %s", cudaGetErrorString(e));
  return OFD_OK;
}

int ofd_group_eligible(ofd_handle *h) {
  if (!h) return fail(OFD_EINVAL, "null handle");
  return (h->s.nks > 0 && h->be->tiled_ok(h->s)) ? 1 : 0;
}

int ofd_group_step(ofd_group *g, int nsteps) {
  if (!g) return fail(OFD_EINVAL, "null group");
  if (nsteps < 0) return fail(OFD_EINVAL, "nsteps < 0");
  if (nsteps == 0) return OFD_OK;
  const int n = (int)g->members.size();
  // members' earlier work (uploads, own steps) comes first
  for (int i = 0; i < n; ++i) {
    OFD_CUDA(cudaEventRecord(g->ready[i], g->members[i]->stream));
    OFD_CUDA(cudaStreamWaitEvent(g->stream, g->ready[i], 0));
  }
  int done = 0;
  while (nsteps - done >= 2) {
    const int p = (int)(g->steps & 1);
    if (!g->graph2[p]) {
      cudaGraph_t gr = nullptr;
      OFD_CUDA(cudaStreamBeginCapture(g->stream, cudaStreamCaptureModeThreadLocal));
      g->be->group_step(g->plan, p, g->stream);
      g->be->group_step(g->plan, 1 - p, g->stream);
      cudaError_t e = cudaStreamEndCapture(g->stream, &gr);
      if (e != cudaSuccess) return fail(OFD_ECUDA, "group graph capture failed: %s", cudaGetErrorString(e));
      e = cudaGraphInstantiate(&g->graph2[p], gr, 0);
      cudaGraphDestroy(gr);
      if (e != cudaSuccess) return fail(OFD_ECUDA, "group graph instantiation failed: %s", cudaGetErrorString(e));
    }
    OFD_CUDA(cudaGraphLaunch(g->graph2[p], g->stream));
    g->steps += 2;
    done += 2;
  }
  if (done < nsteps) {
    g->be->group_step(g->plan, (int)(g->steps & 1), g->stream);
    g->steps += 1;
  }
  OFD_CUDA(cudaGetLastError());
  // later work on a member's own stream comes after the group's
  OFD_CUDA(cudaEventRecord(g->done, g->stream));
  for (int i = 0; i < n; ++i) {
    OFD_CUDA(cudaStreamWaitEvent(g->members[i]->stream, g->done, 0));
    g->members[i]->steps += nsteps;
  }
  return OFD_OK;
}

int ofd_group_query(ofd_group *g) {
  if (!g) return fail(OFD_EINVAL, "null group");
  const cudaError_t e = cudaStreamQuery(g->stream);
  if (e == cudaSuccess) return 0;
  if (e == cudaErrorNotReady) return 1;
  return fail(OFD_ECUDA, "cudaStreamQuery: %s", cudaGetErrorString(e));
}

int ofd_group_sync(ofd_group *g) {
  if (!g) return fail(OFD_EINVAL, "null group");
  OFD_CUDA(cudaStreamSynchronize(g->stream));
  for (ofd_handle *h : g->members) {
    const int rc = check_err_word(h);
    if (rc) return rc;
  }
  return OFD_OK;
}

int ofd_query(ofd_handle *h) {
  if (!h) return fail(OFD_EINVAL, "null handle");
  const cudaError_t e = cudaStreamQuery(h->stream);
  if (e == cudaSuccess) return 0;
  if (e == cudaErrorNotReady) return 1;
  return fail(OFD_ECUDA, "cudaStreamQuery: %s", cudaGetErrorString(e));
}

int ofd_sync(ofd_handle *h) {
  if (!h) return fail(OFD_EINVAL, "null handle");
  OFD_CUDA(cudaStreamSynchronize(h->stream));
  return check_err_word(h);
}

int ofd_field_sumsq(ofd_handle *h, int level, double out[9]) {
  if (!h || !out) return fail(OFD_EINVAL, "null argument");
  if (level < 0 || level > 1) return fail(OFD_EINVAL, "bad level %d", level);
  h->be->sumsq(h->s, level, h->d_out, h->stream);
  OFD_CUDA(cudaGetLastError());
  OFD_CUDA(cudaMemcpyAsync(out, h->d_out, sizeof(double) * NF, cudaMemcpyDeviceToHost, h->stream));
  OFD_CUDA(cudaStreamSynchronize(h->stream));
  return OFD_OK;
}

int ofd_field_absmax(ofd_handle *h, int level, double out[9]) {
  if (!h || !out) return fail(OFD_EINVAL, "null argument");
  if (level < 0 || level > 1) return fail(OFD_EINVAL, "bad level %d", level);
  h->be->absmax(h->s, level, h->d_out, h->stream);
  OFD_CUDA(cudaGetLastError());
  OFD_CUDA(cudaMemcpyAsync(out, h->d_out, sizeof(double) * NF, cudaMemcpyDeviceToHost, h->stream));
  OFD_CUDA(cudaStreamSynchronize(h->stream));
  return OFD_OK;
}

int ofd_field_view_get(ofd_handle *h, int field, int level, ofd_field_view *out) {
  int rc = check_fl(h, field, level);
  if (rc) return rc;
  if (!out) return fail(OFD_EINVAL, "null out");
  out->base = (char *)h->s.field[field] + (size_t)level * h->s.g.level * h->s.esize;
  out->pitch = h->s.g.P;
  out->storage = h->s.storage;
  out->scale = h->s.scale[field];
  return OFD_OK;
}

}  // extern "C"
