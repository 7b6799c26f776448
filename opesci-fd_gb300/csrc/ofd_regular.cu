// Regular-grid (acoustic) scheme: one field on three time levels, updated by
// the sum-of-products expression RegularGrid emits for a second-order-in-time
// equation (opesci/regulargrid.py:592-619 kernel_sympy/simple_kernel; time
// loop opesci/templates/regular3d_tmpl.py:94-105; level rotation
// regulargrid.py:408-433: _t0 = _ti % 3, _t1 = (_t0+1) % 3, _t2 = (_t1+1) % 3,
// u[_t2] = f(u[_t1], u[_t0]) on the interior, margins never written).
//
// HBM-bound: per interior point the sweep reads u[t] and u[t-1] once and
// writes u[t+1] once (12 B/LUP in FP32).  Two variants: a direct one (the
// default, below) and a shared-memory ring.  In both a CTA owns a 32(z) x
// 8(y) column tile and walks a chunk of x planes.  In the ring variant,
// level t is staged in a shared-memory
// ring of 2R+1 planes of the tile plus an R-wide halo, so each value of u[t]
// is read from memory once per CTA and every stencil term of the table is a
// shared-memory read; level t-1 terms read global memory directly.  Terms
// are evaluated in table order as acc = c0*v0, acc = acc + ck*vk with
// round-to-nearest multiplies and adds and no contraction, the rounding of
// the reference's left-to-right C expression.
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>

#include <cuda_runtime.h>

#include "ofd.h"

namespace ofd {
int fail_msg(int code, const char *msg);   // ofd_runtime.cu: sets ofd_last_error()
}

namespace {

int rfail(int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  return ofd::fail_msg(code, buf);
}

#define REG_CUDA(call)                                                                        \
  do {                                                                                        \
    cudaError_t _e = (call);                                                                  \
    if (_e != cudaSuccess)                                                                    \
      return rfail(OFD_ECUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(_e), __FILE__, \
                   __LINE__);                                                                 \
  } while (0)

constexpr int TZ = 32;            // tile width along z (one warp)
constexpr int TY = 8;             // tile height along y (eight warps)
constexpr int NT = TZ * TY;       // threads per CTA
constexpr int MAX_MARGIN = 8;     // space order 16
constexpr int MAXE = 8;           // ring elements per thread per plane: (32+2R)(8+2R) <= 8*256

template <typename T>
struct RegSweep {
  const T *cur;    // level t, element (x,y,z) at cur[x*plane + y*P + z]
  const T *prev;   // level t-1
  T *next;         // level t+1
  int n1, n2, n3, m;
  int P, plane;
  int chunk;       // x planes per CTA
  int nterms;
  signed char lvl[OFD_REGULAR_MAX_TERMS];
  signed char dx[OFD_REGULAR_MAX_TERMS];
  short soff[OFD_REGULAR_MAX_TERMS];   // (dy+R)*(32+2R) + dz+R within a ring plane
  int goff[OFD_REGULAR_MAX_TERMS];     // dx*plane + dy*P + dz
  T coef[OFD_REGULAR_MAX_TERMS];
};

__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }

template <typename T>
__global__ void __launch_bounds__(NT) regular_sweep_kernel(const RegSweep<T> a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int R = a.m, NP = 2 * R + 1, W = TZ + 2 * R, H = TY + 2 * R, PS = W * H;
  T *ring = reinterpret_cast<T *>(smem);
  int *slot = reinterpret_cast<int *>(ring + NP * PS);

  const int tid = threadIdx.y * TZ + threadIdx.x;
  const int zt = a.m + blockIdx.x * TZ, yt = a.m + blockIdx.y * TY;
  const int xb = a.m + blockIdx.z * a.chunk;
  const int xe = min(xb + a.chunk, a.n1 - a.m);

  // the ring elements this thread stages, as offsets within an x plane of
  // the level (-1: outside the array, staged as zero; never read by an
  // interior point's term since offsets are bounded by the margin)
  int src[MAXE];
#pragma unroll
  for (int i = 0; i < MAXE; ++i) {
    const int e = tid + i * NT;
    src[i] = -1;
    if (e < PS) {
      const int r = e / W, c = e - r * W;
      const int yy = yt - R + r, zz = zt - R + c;   // >= 0: the tile starts at the margin
      if (yy < a.n2 && zz < a.n3) src[i] = yy * a.P + zz;
    }
  }
  auto stage = [&](int x) {   // plane x of level t into its ring slot
    T *dst = ring + (x % NP) * PS;
    const T *plane = a.cur + (long)x * a.plane;
#pragma unroll
    for (int i = 0; i < MAXE; ++i) {
      const int e = tid + i * NT;
      if (e < PS) dst[e] = src[i] >= 0 ? plane[src[i]] : T(0);
    }
  };

  for (int x = xb - R; x < xb + R; ++x) stage(x);   // planes xb-R .. xb+R-1, all inside [0, n1)

  const int y = yt + threadIdx.y, z = zt + threadIdx.x;
  const bool active = y < a.n2 - a.m && z < a.n3 - a.m;
  const int me = threadIdx.y * W + threadIdx.x;
  for (int x = xb; x < xe; ++x) {
    stage(x + R);
    if (tid < NP) slot[tid] = ((x - R + tid) % NP) * PS;
    __syncthreads();
    if (active) {
      const long g = (long)x * a.plane + (long)y * a.P + z;
      T acc = T(0);
#pragma unroll 4
      for (int k = 0; k < a.nterms; ++k) {
        const T v = a.lvl[k] ? ring[slot[a.dx[k] + R] + me + a.soff[k]] : a.prev[g + a.goff[k]];
        const T p = mul_rn(a.coef[k], v);
        acc = k ? add_rn(acc, p) : p;
      }
      a.next[g] = acc;
    }
    __syncthreads();   // the next stage() overwrites the slot of plane x-R
  }
}

// Direct variant: no shared memory and no barriers.  Each thread walks a
// chunk of x planes of one (y, z) column and reads every term through the
// read-only path; neighbours along z and y come from the same or nearby
// warps' lines in L1, neighbours along x from planes this thread read a few
// iterations earlier, so memory traffic stays near the algorithmic 12 B/LUP
// while every warp is independent.  The thread advances XU planes at a time:
// for each term it loads the XU planes' values before the XU multiply-adds,
// so XU times as many independent loads (and DRAM misses: the leading plane
// of level t and level t-1) are in flight per warp; each point's chain keeps
// the table order, so results are those of one plane at a time.  Measured
// at 512^3 FP32: XU = 1 / 4 / 8 / 16 gave 209 / 367 / 426 / 416 GLUP/s at
// space order 4 and 134 / 223 / 275 / 294 at space order 8; the launch
// takes 8 for margins up to 2 and 16 above.
template <typename T, int XU>
__global__ void __launch_bounds__(NT) regular_direct_kernel(const RegSweep<T> a) {
  const int z = a.m + blockIdx.x * TZ + threadIdx.x;
  const int y = a.m + blockIdx.y * TY + threadIdx.y;
  if (z >= a.n3 - a.m || y >= a.n2 - a.m) return;
  const int xb = a.m + blockIdx.z * a.chunk;
  const int xe = min(xb + a.chunk, a.n1 - a.m);
  const T *__restrict__ cur = a.cur;
  const T *__restrict__ prev = a.prev;
  T *__restrict__ next = a.next;
  const long pl = a.plane;
  long g = (long)xb * pl + (long)y * a.P + z;
  int x = xb;
  for (; x + XU <= xe; x += XU, g += XU * pl) {
    T acc[XU];
#pragma unroll 4
    for (int k = 0; k < a.nterms; ++k) {
      const T *p = (a.lvl[k] ? cur : prev) + g + a.goff[k];
      T v[XU];
#pragma unroll
      for (int u = 0; u < XU; ++u) v[u] = __ldg(p + u * pl);
      const T c = a.coef[k];
#pragma unroll
      for (int u = 0; u < XU; ++u) {
        const T q = mul_rn(c, v[u]);
        acc[u] = k ? add_rn(acc[u], q) : q;
      }
    }
#pragma unroll
    for (int u = 0; u < XU; ++u) next[g + u * pl] = acc[u];
  }
  for (; x < xe; ++x, g += pl) {
    T acc = T(0);
#pragma unroll 8
    for (int k = 0; k < a.nterms; ++k) {
      const T *base = a.lvl[k] ? cur : prev;
      const T p = mul_rn(a.coef[k], __ldg(base + g + a.goff[k]));
      acc = k ? add_rn(acc, p) : p;
    }
    next[g] = acc;
  }
}

size_t esize_of(int storage) { return storage == OFD_F64 ? 8 : storage == OFD_F32 ? 4 : 0; }

size_t ring_bytes(int m, size_t es) {
  const size_t PS = (size_t)(TZ + 2 * m) * (TY + 2 * m);
  return (2 * m + 1) * PS * es + sizeof(int) * (2 * m + 1);
}

}  // namespace

struct ofd_regular {
  ofd_regular_config cfg;
  cudaStream_t stream = nullptr;
  void *raw = nullptr;
  size_t es = 4;
  int z0 = 0;          // element offset of z = 0 inside a padded row
  int P = 0;           // row pitch (elements)
  long plane = 0;      // elements per x plane
  long level = 0;      // elements per level (256-B multiple)
  long ti = 0;         // steps done
  int chunk = 8;
  int variant = 0;     // 0: direct, 1: shared-memory ring
  dim3 grid;
  size_t smem = 0;
  RegSweep<float> a32[3];    // by ti % 3
  RegSweep<double> a64[3];
};

namespace {

template <typename T>
T *level_ptr(ofd_regular *h, int l) {
  return reinterpret_cast<T *>(h->raw) + (long)l * h->level + h->z0;
}

template <typename T>
void fill_args(ofd_regular *h, RegSweep<T> *out) {
  const ofd_regular_config &c = h->cfg;
  const int R = c.margin, W = TZ + 2 * R;
  for (int r = 0; r < 3; ++r) {
    RegSweep<T> &a = out[r];
    memset(&a, 0, sizeof(a));
    const int t0 = r, t1 = (t0 + 1) % 3, t2 = (t1 + 1) % 3;
    a.cur = level_ptr<T>(h, t1);
    a.prev = level_ptr<T>(h, t0);
    a.next = level_ptr<T>(h, t2);
    a.n1 = c.dim[0];
    a.n2 = c.dim[1];
    a.n3 = c.dim[2];
    a.m = R;
    a.P = h->P;
    a.plane = (int)h->plane;
    a.chunk = h->chunk;
    a.nterms = c.nterms;
    for (int k = 0; k < c.nterms; ++k) {
      const int dx = c.offset[k][0], dy = c.offset[k][1], dz = c.offset[k][2];
      a.lvl[k] = (signed char)c.level[k];
      a.dx[k] = (signed char)dx;
      a.soff[k] = (short)((dy + R) * W + dz + R);
      a.goff[k] = (int)(dx * h->plane + (long)dy * h->P + dz);
      a.coef[k] = (T)c.coef[k];
    }
  }
}

int check(const ofd_regular_config *c) {
  if (!c) return rfail(OFD_EINVAL, "null config");
  if (esize_of(c->storage) == 0) return rfail(OFD_EINVAL, "regular scheme storage must be OFD_F32 or OFD_F64");
  if (c->margin < 1 || c->margin > MAX_MARGIN)
    return rfail(OFD_EINVAL, "margin %d outside [1, %d]", c->margin, MAX_MARGIN);
  for (int i = 0; i < 3; ++i) {
    if (c->dim[i] < 2 * c->margin + 1) return rfail(OFD_EINVAL, "dim%d = %d has no interior", i + 1, c->dim[i]);
    if (c->dim[i] > (1 << 15)) return rfail(OFD_EINVAL, "dim%d = %d too large", i + 1, c->dim[i]);
  }
  if (c->variant < 0 || c->variant > 1) return rfail(OFD_EINVAL, "variant %d outside [0, 1]", c->variant);
  if (c->nterms < 1 || c->nterms > OFD_REGULAR_MAX_TERMS)
    return rfail(OFD_EINVAL, "nterms %d outside [1, %d]", c->nterms, OFD_REGULAR_MAX_TERMS);
  for (int k = 0; k < c->nterms; ++k) {
    if (c->level[k] != 0 && c->level[k] != 1) return rfail(OFD_EINVAL, "term %d: level must be 0 or 1", k);
    for (int d = 0; d < 3; ++d)
      if (c->offset[k][d] < -c->margin || c->offset[k][d] > c->margin)
        return rfail(OFD_EINVAL, "term %d: offset %d on axis %d exceeds the margin %d", k, c->offset[k][d], d,
                     c->margin);
  }
  return OFD_OK;
}

int copy_level(ofd_regular *h, int level, const void *src, void *dst, cudaMemcpyKind kind, bool to_dev) {
  if (!h) return rfail(OFD_EINVAL, "null handle");
  if (level < 0 || level > 2) return rfail(OFD_EINVAL, "level %d outside [0, 2]", level);
  if (to_dev ? !src : !dst) return rfail(OFD_EINVAL, "null array");
  const size_t row = (size_t)h->cfg.dim[2] * h->es, pitch = (size_t)h->P * h->es;
  const size_t rows = (size_t)h->cfg.dim[0] * h->cfg.dim[1];
  unsigned char *lv = reinterpret_cast<unsigned char *>(h->raw) + ((size_t)level * h->level + h->z0) * h->es;
  if (to_dev)
    REG_CUDA(cudaMemcpy2DAsync(lv, pitch, src, row, row, rows, kind, h->stream));
  else
    REG_CUDA(cudaMemcpy2DAsync(dst, row, lv, pitch, row, rows, kind, h->stream));
  REG_CUDA(cudaStreamSynchronize(h->stream));
  return OFD_OK;
}

}  // namespace

// The ring sweep's dynamic shared memory limit (a per-function, per-device
// attribute shared by every handle): raised to the largest ring a handle of
// this process has needed so far on the current device, never lowered, so
// handles of different margins coexist; the direct sweep uses none.
static cudaError_t raise_ring_limit(size_t es, size_t bytes) {
  static std::mutex mu;
  static size_t set_f32[64] = {}, set_f64[64] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) dev = 63;
  std::lock_guard<std::mutex> lock(mu);
  size_t &cur = es == 4 ? set_f32[dev] : set_f64[dev];
  if (bytes <= cur) return cudaSuccess;
  e = es == 4 ? cudaFuncSetAttribute(regular_sweep_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes)
              : cudaFuncSetAttribute(regular_sweep_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)bytes);
  if (e == cudaSuccess) cur = bytes;
  return e;
}

extern "C" {

int ofd_regular_create(const ofd_regular_config *cfg, ofd_regular **out) {
  if (!out) return rfail(OFD_EINVAL, "null out");
  *out = nullptr;
  int rc = check(cfg);
  if (rc) return rc;
  ofd_regular *h = new ofd_regular();
  h->cfg = *cfg;
  h->es = esize_of(cfg->storage);
  const int m = cfg->margin;
  const int A = (int)(128 / h->es);   // elements per 128-B line
  h->z0 = (A - m % A) % A;            // interior z = m starts a 128-B line: tile rows are line-aligned
  h->P = (h->z0 + cfg->dim[2] + A - 1) / A * A;
  h->plane = (long)cfg->dim[1] * h->P;
  if (h->plane * (2 * m + 1) >= (1L << 31)) {
    delete h;
    return rfail(OFD_EINVAL, "x plane of %ld elements too large", h->plane);
  }
  const long al = (long)(256 / h->es);
  h->level = ((long)cfg->dim[0] * h->plane + al - 1) / al * al;
  const int nx = cfg->dim[0] - 2 * m, ny = cfg->dim[1] - 2 * m, nz = cfg->dim[2] - 2 * m;
  const long tiles = (long)((nz + TZ - 1) / TZ) * ((ny + TY - 1) / TY);
  h->variant = cfg->variant;
  long chunk;
  if (h->variant == 0) {
    // short columns: x neighbours are still in L1 when a thread reaches them
    chunk = 16;
  } else {
    // about eight waves of 8 resident CTAs on each of the GPU's SMs
    int sms = 152;
    int dev = 0;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long want = (long)sms * 8 * 8;
    chunk = ((long)nx * tiles + want - 1) / want;
    if (chunk < 8) chunk = 8;
  }
  if (chunk > nx) chunk = nx;
  h->chunk = (int)chunk;
  h->grid = dim3((nz + TZ - 1) / TZ, (ny + TY - 1) / TY, (nx + h->chunk - 1) / h->chunk);
  h->smem = h->variant == 1 ? ring_bytes(m, h->es) : 0;
  cudaError_t e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc(&h->raw, (size_t)h->level * 3 * h->es);
  if (e == cudaSuccess) e = cudaMemsetAsync(h->raw, 0, (size_t)h->level * 3 * h->es, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  if (e == cudaSuccess && h->variant == 1) e = raise_ring_limit(h->es, h->smem);
  if (e != cudaSuccess) {
    const int code = e == cudaErrorMemoryAllocation ? OFD_ENOMEM : OFD_ECUDA;
    if (h->raw) cudaFree(h->raw);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return rfail(code, "ofd_regular_create: %s", cudaGetErrorString(e));
  }
  if (h->es == 4)
    fill_args<float>(h, h->a32);
  else
    fill_args<double>(h, h->a64);
  *out = h;
  return OFD_OK;
}

int ofd_regular_destroy(ofd_regular *h) {
  if (!h) return OFD_OK;
  if (h->stream) cudaStreamSynchronize(h->stream);
  if (h->raw) cudaFree(h->raw);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return OFD_OK;
}

int ofd_regular_upload(ofd_regular *h, int level, const void *host) {
  return copy_level(h, level, host, nullptr, cudaMemcpyHostToDevice, true);
}
int ofd_regular_download(ofd_regular *h, int level, void *host) {
  return copy_level(h, level, nullptr, host, cudaMemcpyDeviceToHost, false);
}
int ofd_regular_upload_device(ofd_regular *h, int level, const void *dev) {
  return copy_level(h, level, dev, nullptr, cudaMemcpyDeviceToDevice, true);
}
int ofd_regular_download_device(ofd_regular *h, int level, void *dev) {
  return copy_level(h, level, nullptr, dev, cudaMemcpyDeviceToDevice, false);
}

int ofd_regular_step(ofd_regular *h, int nsteps) {
  if (!h) return rfail(OFD_EINVAL, "null handle");
  if (nsteps < 0) return rfail(OFD_EINVAL, "nsteps must be >= 0");
  for (int s = 0; s < nsteps; ++s, ++h->ti) {
    const int r = (int)(h->ti % 3);
    if (h->variant == 0) {
      const bool wide = h->cfg.margin > 2;
      if (h->es == 4) {
        if (wide) regular_direct_kernel<float, 16><<<h->grid, dim3(TZ, TY), 0, h->stream>>>(h->a32[r]);
        else regular_direct_kernel<float, 8><<<h->grid, dim3(TZ, TY), 0, h->stream>>>(h->a32[r]);
      } else {
        if (wide) regular_direct_kernel<double, 16><<<h->grid, dim3(TZ, TY), 0, h->stream>>>(h->a64[r]);
        else regular_direct_kernel<double, 8><<<h->grid, dim3(TZ, TY), 0, h->stream>>>(h->a64[r]);
      }
    } else {
      if (h->es == 4)
        regular_sweep_kernel<float><<<h->grid, dim3(TZ, TY), h->smem, h->stream>>>(h->a32[r]);
      else
        regular_sweep_kernel<double><<<h->grid, dim3(TZ, TY), h->smem, h->stream>>>(h->a64[r]);
    }
    REG_CUDA(cudaGetLastError());
  }
  return OFD_OK;
}

int ofd_regular_step_timed(ofd_regular *h, int nsteps, double *ms) {
  if (!h || !ms) return rfail(OFD_EINVAL, "null argument");
  cudaEvent_t a = nullptr, b = nullptr;
  REG_CUDA(cudaEventCreate(&a));
  cudaError_t e = cudaEventCreate(&b);
  if (e == cudaSuccess) e = cudaEventRecord(a, h->stream);
  int rc = OFD_OK;
  if (e == cudaSuccess) {
    rc = ofd_regular_step(h, nsteps);
    if (rc == OFD_OK) e = cudaEventRecord(b, h->stream);
  }
  float f = 0.f;
  if (e == cudaSuccess && rc == OFD_OK) e = cudaEventSynchronize(b);
  if (e == cudaSuccess && rc == OFD_OK) e = cudaEventElapsedTime(&f, a, b);
  cudaEventDestroy(a);
  if (b) cudaEventDestroy(b);
  if (rc != OFD_OK) return rc;
  if (e != cudaSuccess) return rfail(OFD_ECUDA, "event timing: %s", cudaGetErrorString(e));
  *ms = f;
  return OFD_OK;
}

int ofd_regular_get_step(ofd_regular *h, long *steps) {
  if (!h || !steps) return rfail(OFD_EINVAL, "null argument");
  *steps = h->ti;
  return OFD_OK;
}

int ofd_regular_set_step(ofd_regular *h, long steps) {
  if (!h) return rfail(OFD_EINVAL, "null handle");
  if (steps < 0) return rfail(OFD_EINVAL, "steps must be >= 0");
  h->ti = steps;
  return OFD_OK;
}

int ofd_regular_sync(ofd_regular *h) {
  if (!h) return rfail(OFD_EINVAL, "null handle");
  REG_CUDA(cudaStreamSynchronize(h->stream));
  return OFD_OK;
}

void *ofd_regular_stream(ofd_regular *h) { return h ? (void *)h->stream : nullptr; }

}  // extern "C"
