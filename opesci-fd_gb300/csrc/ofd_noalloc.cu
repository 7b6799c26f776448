// Allocation-free FP64 sum of squares of one field.
//
// ofd_field_sumsq reduces through a scratch buffer that ofd_create allocates
// with the handle.  Some callers cannot allocate device memory at all: code
// that runs while a CUDA graph is being captured (cudaMalloc and cudaFree are
// not capturable and synchronise the device), plugins that live inside
// another framework's memory pool and must not grow the process's footprint,
// and serving loops that must not stall on an allocator.  They pass their own
// input and output buffers to ofd_sumsq_field_noalloc and the partial sums go
// to the fixed array below instead of a per-call allocation.
//
// The scratch is one double per x plane, so the call accepts at most
// OFD_NOALLOC_MAX_PLANES planes and rejects larger grids.  Every GPU that
// loads this library holds the 32 KB array until the process exits.  Every
// call shares it and each call overwrites the entries it uses, so two calls
// whose kernels overlap on the GPU (different streams, no ordering between
// them) race on it; callers must serialise them.
//
// The array's device address belongs to the CUDA context that is current
// when the call is made.  A call outside stream capture looks it up afresh
// and records it for that context; a call on a capturing stream (where the
// lookup may not be made) uses the address recorded for its context and
// fails if there is none.  After cudaDeviceReset the context is new, so the
// first call after a reset must again come before any capture.
#include <climits>
#include <cstdio>
#include <mutex>
#include <string>

#include <cuda.h>

#include "ofd.h"

#define OFD_NOALLOC_MAX_PLANES 4096
#define OFD_NOALLOC_MAX_CONTEXTS 64

static __device__ __align__(256) double g_noalloc_partial[OFD_NOALLOC_MAX_PLANES];

namespace {

std::mutex g_setup_mutex;
// scratch addresses by context (recorded by calls outside capture)
CUcontext g_ctx[OFD_NOALLOC_MAX_CONTEXTS] = {};
double *g_ctx_ptr[OFD_NOALLOC_MAX_CONTEXTS] = {};
thread_local std::string g_noalloc_error;

typedef CUresult (*CtxGetCurrentFn)(CUcontext *);

// cuCtxGetCurrent through the runtime's driver entry point (the library does
// not link libcuda itself)
CtxGetCurrentFn ctx_get_current() {
  static CtxGetCurrentFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (CtxGetCurrentFn)p;
  });
  return fn;
}

int noalloc_fail(int code, const char *msg) {
  g_noalloc_error = msg;
  return code;
}

// One CTA per x plane: FP64 sum of squares over the plane's interior rows,
// written to the plane's scratch entry (no atomics: the result does not depend
// on scheduling).
__global__ void plane_sumsq(const float *__restrict__ f, int n1, int n2, int n3, int m, double *partial) {
  const int x = blockIdx.x + m;
  const long plane = (long)n2 * n3;
  double acc = 0;
  const long ny = n2 - 2 * m, nz = n3 - 2 * m;
  for (long i = threadIdx.x; i < ny * nz; i += blockDim.x) {
    const long y = m + i / nz, z = m + i % nz;
    const double v = f[(long)x * plane + y * n3 + z];
    acc += v * v;
  }
  __shared__ double sh[256];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

__global__ void planes_total(const double *partial, int nplanes, double *out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double a = 0;
    for (int i = 0; i < nplanes; ++i) a += partial[i];
    *out = a;
  }
}

}  // namespace

extern "C" {

const char *ofd_noalloc_last_error(void) { return g_noalloc_error.c_str(); }

int ofd_sumsq_field_noalloc(const float *field, const int dims[3], int margin, double *out, void *stream) {
  if (!field || !dims || !out) return noalloc_fail(OFD_EINVAL, "null argument");
  if (margin < 0 || dims[0] <= 2 * margin || dims[1] <= 2 * margin || dims[2] <= 2 * margin)
    return noalloc_fail(OFD_EINVAL, "dims must exceed twice the margin");
  const int nplanes = dims[0] - 2 * margin;
  if (nplanes > OFD_NOALLOC_MAX_PLANES) {
    char buf[160];
    snprintf(buf, sizeof(buf), "%d interior planes exceed the fixed scratch of %d planes", nplanes,
             OFD_NOALLOC_MAX_PLANES);
    return noalloc_fail(OFD_EINVAL, buf);
  }
  if ((long)(dims[1] - 2 * margin) * (dims[2] - 2 * margin) > INT_MAX)
    return noalloc_fail(OFD_EINVAL, "an x plane holds more than 2^31 - 1 interior points");
  cudaStream_t st = (cudaStream_t)stream;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  cudaError_t ce = cudaStreamIsCapturing(st, &cap);
  if (ce != cudaSuccess) {
    g_noalloc_error = std::string("cudaStreamIsCapturing failed: ") + cudaGetErrorString(ce);
    return OFD_ECUDA;
  }
  CtxGetCurrentFn get_ctx = ctx_get_current();
  CUcontext ctx = nullptr;
  if (!get_ctx || get_ctx(&ctx) != CUDA_SUCCESS || !ctx)
    return noalloc_fail(OFD_ECUDA, "no current CUDA context");
  double *partial = nullptr;
  {
    // the device address of the scratch array in this context (the host-side
    // symbol is only a stand-in and must not reach a kernel)
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    int slot = -1, free_slot = -1;
    for (int i = 0; i < OFD_NOALLOC_MAX_CONTEXTS; ++i) {
      if (g_ctx[i] == ctx) slot = i;
      if (!g_ctx[i] && free_slot < 0) free_slot = i;
    }
    if (cap == cudaStreamCaptureStatusNone) {
      void *p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_partial);
      if (e != cudaSuccess || !p) {
        g_noalloc_error = std::string("cudaGetSymbolAddress failed: ") + cudaGetErrorString(e);
        return OFD_ECUDA;
      }
      if (slot < 0) slot = free_slot;
      if (slot < 0) return noalloc_fail(OFD_EINVAL, "more CUDA contexts than the address table holds");
      g_ctx[slot] = ctx;
      g_ctx_ptr[slot] = (double *)p;
    } else if (slot < 0) {
      return noalloc_fail(OFD_ESTATE,
                          "first call in this CUDA context is on a capturing stream; make one call before capture");
    }
    partial = g_ctx_ptr[slot];
  }
  plane_sumsq<<<nplanes, 256, 0, st>>>(field, dims[0], dims[1], dims[2], margin, partial);
  planes_total<<<1, 32, 0, st>>>(partial, nplanes, out);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    g_noalloc_error = std::string("launch failed: ") + cudaGetErrorString(e);
    return OFD_ECUDA;
  }
  return OFD_OK;
}

}  // extern "C"
