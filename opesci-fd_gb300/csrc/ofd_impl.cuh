// Backend: the kernel launches of one (radius R, storage S) instantiation.
// The runtime (ofd_runtime.cu) owns the handle and memory; each
// ofd_inst_*.cu file instantiates Impl<R, S> for one storage type so the
// variants compile in parallel.
#pragma once
#include <algorithm>
#include <cstring>
#include <vector>
#include "ofd_common.cuh"
#include "ofd_sweep_plain.cuh"
#include "ofd_sweep_tiled.cuh"
#include "ofd_bc.cuh"
#include "ofd_persistent.cuh"

namespace ofd {

struct DevState {
  Geom g;
  int z0;
  int storage;
  size_t esize;
  int R;
  void *field[NF];     // field f, level 0, element (0,0,0) (z0 applied)
  float *media[NM];    // media array, element (0,0,0) (z0 applied)
  float scale[NF];
  int face[6];
  int legacy;
  double dt, h[3], c[4];
  long src_off;        // -1: no source
  float *d_wav;
  int nt;
  int variant;         // 0 best, 1 plain
  double *d_partial;   // reduction scratch (>= 2048 doubles)
  long *d_step;        // device step counter (graph-safe source index)
  // receivers: element offsets (in a level) and a trace buffer
  // traces[step][k][r], k = U V W P with P = (Txx + Tyy + Tzz) / 3
  int nrec, rec_cap;
  long *d_rec;
  float *d_traces;
  TiledCtx tiled;      // TMA descriptors for the tiled sweeps
  // launch tuning (autotuner knobs): per-sweep variant 0 tiled / 1 plain,
  // target waves for the x chunking, plain-kernel block shape
  int var_stress, var_velocity, chunk_waves, plain_bx, plain_by;
  int persistent;      // 1: time steps run in one cooperative launch
  unsigned *d_bar;     // grid-barrier words of the persistent kernel
  int het;             // 1: media arrays are factors of the update (read mode)
  int sr;              // 16-bit storage: stochastic rounding of the sweeps' stores
  int gen_ghost;       // space order 4: generated Levander ghost expressions (literals d_kg)
  float *d_kg;
  // precomputed normal-stress recompute values (generated ghosts): 12 planes
  // of rcs floats.  rc_mode 0: computed on the handle's stream after the
  // stress sweep; 1: on stream st2 (highest priority) beside the sweep.
  // rc_bps: blocks of 128 threads per SM of the recompute grid.
  float *d_rc;
  long rcs;
  int rc_mode, rc_bps;
  cudaStream_t st2;
  cudaEvent_t ev_fork, ev_join;
  int nks, nkv;        // literal-table sizes (0 until ofd_set_coefficients)
  float Ks[OFD_MAX_K], Kv[OFD_MAX_K];
};

struct GroupPlanBase {
  virtual ~GroupPlanBase() {}
};

// Optional per-kernel-class events of a profiled step: ev[2k], ev[2k+1]
// bracket class k (0 stress sweep, 1 stress ghosts, 2 velocity sweep,
// 3 velocity ghosts + source).
struct StepEvents {
  cudaEvent_t ev[8];
};

struct Backend {
  virtual ~Backend() {}
  virtual void step(const DevState &s, int t0, cudaStream_t st, const StepEvents *ev = nullptr) = 0;
  virtual int launches_per_step(const DevState &s) const = 0;
  virtual void boundary_init(const DevState &s, int level, cudaStream_t st) = 0;
  virtual void to_padded(const DevState &s, const float *dense, int f, int level, cudaStream_t st) = 0;
  virtual void from_padded(const DevState &s, float *dense, int f, int level, cudaStream_t st) = 0;
  virtual void sumsq(const DevState &s, int level, double *d_out9, cudaStream_t st) = 0;
  virtual void absmax(const DevState &s, int level, double *d_out9, cudaStream_t st) = 0;
  // one-time launch attributes (dynamic shared memory) so that later launches
  // can be captured into graphs
  virtual void prepare(const DevState &s) = 0;
  // nsteps whole steps in one cooperative launch starting at parity p0;
  // returns a cudaError_t
  virtual int step_persistent(const DevState &s, int p0, int nsteps, cudaStream_t st) = 0;
  // literal-table sizes of the generated expressions for media mode het
  virtual int table_size(int het, int stress) const = 0;
  // literal-table size of the generated ghost expressions (0: none for this
  // space order and storage)
  virtual int ghost_table_size(int het) const = 0;
  // Grouped stepping: device tables of the members' arguments (all members
  // share this backend's space order and storage, and one media mode), and
  // one step of every member in 8 grouped launches.  chunk_planes: x chunk
  // length of the members' sweep CTAs.  The tables are allocated and filled
  // in stream order on st (no device-wide synchronisation) and freed the
  // same way when the plan is deleted.  group_build returns nullptr and sets
  // *cuda_err on a CUDA failure.
  virtual GroupPlanBase *group_build(const DevState *const *members, int n, int chunk_planes, cudaStream_t st,
                                     cudaError_t *cuda_err) = 0;
  virtual void group_step(GroupPlanBase *plan, int t0, cudaStream_t st) = 0;
  // the handle's sweeps can run tiled (a group member must)
  virtual bool tiled_ok(const DevState &s) const = 0;
  // the handle's literal table of a sweep repeats its values as KMap says
  virtual bool kmap_ok(const DevState &s, bool stress) const = 0;
};

// One backend per (storage, radius), each defined in its own translation unit:
// ofd_inst_<storage>.cu compiled once per radius with -DOFD_INST_R=1..4, so
// the heavy kernel instantiations build in parallel.
template <typename S, int R> Backend *make_backend();
#define OFD_DECLARE_BACKENDS(S)                  \
  template <> Backend *make_backend<S, 1>();     \
  template <> Backend *make_backend<S, 2>();     \
  template <> Backend *make_backend<S, 3>();     \
  template <> Backend *make_backend<S, 4>();
OFD_DECLARE_BACKENDS(float)
OFD_DECLARE_BACKENDS(double)
OFD_DECLARE_BACKENDS(__half)
OFD_DECLARE_BACKENDS(__nv_bfloat16)

template <typename S>
inline Backend *backend_for(int R) {
  switch (R) {
    case 1: return make_backend<S, 1>();
    case 2: return make_backend<S, 2>();
    case 3: return make_backend<S, 3>();
    case 4: return make_backend<S, 4>();
  }
  return nullptr;
}

// SMs of the current device (cached per device)
inline int sm_count() {
  static int cache[64] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152;
  if (!cache[dev]) {
    int n = 0;
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    cache[dev] = n > 0 ? n : 152;
  }
  return cache[dev];
}

// Default schedule of the generated ghosts' recompute (ofd_set_ghost_schedule)
#define OFD_RC_MODE_DEFAULT 1
#define OFD_RC_BPS_DEFAULT 4

// Numerically lowest (most urgent) stream priority of the current device.
inline int greatest_priority() {
  int least = 0, greatest = 0;
  if (cudaDeviceGetStreamPriorityRange(&least, &greatest) != cudaSuccess) return 0;
  return greatest;
}

// ---- generic kernels ------------------------------------------------------

template <typename S>
__global__ void dense_to_padded(const float *__restrict__ src, S *__restrict__ dst, Geom g, float sc) {
  const long n = (long)g.n1 * g.n2 * g.n3;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const int z = (int)(i % g.n3);
    const long r = i / g.n3;
    const int y = (int)(r % g.n2);
    const int x = (int)(r / g.n2);
    dst[(long)x * g.plane + (long)y * g.P + z] = Storage<S>::store((typename Storage<S>::C)src[i], sc);
  }
}

template <typename S>
__global__ void padded_to_dense(const S *__restrict__ src, float *__restrict__ dst, Geom g, float inv) {
  const long n = (long)g.n1 * g.n2 * g.n3;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const int z = (int)(i % g.n3);
    const long r = i / g.n3;
    const int y = (int)(r % g.n2);
    const int x = (int)(r / g.n2);
    dst[i] = (float)Storage<S>::load(src[(long)x * g.plane + (long)y * g.P + z], inv);
  }
}

// Deterministic FP64 sum of squares over the interior of 9 fields: one block
// row per field, fixed grid, tree reduction, then a single-block pass.
template <typename S>
__global__ void sumsq_partial(DevState s, int level, double *partial) {
  const Geom g = s.g;
  const int f = blockIdx.y;
  const S *p = (const S *)s.field[f] + (long)level * g.level;
  const long nx = g.n1 - 2 * g.m, ny = g.n2 - 2 * g.m, nz = g.n3 - 2 * g.m;
  const long n = nx * ny * nz;
  const float inv = 1.f / s.scale[f];
  double acc = 0;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const int z = (int)(i % nz) + g.m;
    const long r = i / nz;
    const int y = (int)(r % ny) + g.m;
    const int x = (int)(r / ny) + g.m;
    const double v = (double)Storage<S>::load(p[(long)x * g.plane + (long)y * g.P + z], inv);
    acc += v * v;
  }
  __shared__ double sh[256];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[f * gridDim.x + blockIdx.x] = sh[0];
}

// Largest magnitude of each field over the interior of a level (storage
// scaling removed), for choosing 16-bit storage scales.
template <typename S>
__global__ void absmax_partial(DevState s, int level, double *partial) {
  const Geom g = s.g;
  const int f = blockIdx.y;
  const S *p = (const S *)s.field[f] + (long)level * g.level;
  const long nx = g.n1 - 2 * g.m, ny = g.n2 - 2 * g.m, nz = g.n3 - 2 * g.m;
  const long n = nx * ny * nz;
  const float inv = 1.f / s.scale[f];
  double acc = 0;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const int z = (int)(i % nz) + g.m;
    const long r = i / nz;
    const int y = (int)(r % ny) + g.m;
    const int x = (int)(r / ny) + g.m;
    const double v = fabs((double)Storage<S>::load(p[(long)x * g.plane + (long)y * g.P + z], inv));
    acc = v > acc ? v : acc;
  }
  __shared__ double sh[256];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] = sh[threadIdx.x] > sh[threadIdx.x + w] ? sh[threadIdx.x] : sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[f * gridDim.x + blockIdx.x] = sh[0];
}

static __global__ void absmax_final(const double *partial, int nblk, double *out) {
  const int f = threadIdx.x;
  if (f < NF) {
    double a = 0;
    for (int i = 0; i < nblk; ++i) a = partial[f * nblk + i] > a ? partial[f * nblk + i] : a;
    out[f] = a;
  }
}

static __global__ void sumsq_final(const double *partial, int nblk, double *out) {
  const int f = threadIdx.x;
  if (f < NF) {
    double a = 0;
    for (int i = 0; i < nblk; ++i) a += partial[f * nblk + i];
    out[f] = a;
  }
}

// ---- Impl -----------------------------------------------------------------

template <int R, typename S>
struct Impl : Backend {
  typedef typename Storage<S>::C C;

  S *fp(const DevState &s, int f, int lvl) const { return (S *)s.field[f] + (long)lvl * s.g.level; }

  SweepArgs<S> sweep_args(const DevState &s, int t0, bool stress) const {
    SweepArgs<S> a;
    a.g = s.g;
    const int t1 = 1 - t0;
    for (int f = 0; f < NF; ++f) {
      const bool is_v = f < 3;
      // stress sweep reads everything at t0; velocity sweep reads V(t0), T(t1)
      const int lin = stress ? t0 : (is_v ? t0 : t1);
      a.in[f] = fp(s, f, lin);
      a.out[f] = fp(s, f, t1);
      a.sc[f] = s.scale[f];
      a.inv[f] = 1.f / s.scale[f];
    }
    for (int i = 0; i < NM; ++i) a.media[i] = s.media[i];
    a.dt = (C)s.dt;
    a.ih1 = (C)(1.0 / s.h[0]);
    a.ih2 = (C)(1.0 / s.h[1]);
    a.ih3 = (C)(1.0 / s.h[2]);
    for (int k = 0; k < 4; ++k) a.c[k] = (C)s.c[k];
    a.xchunk = 0;
    a.sr = (s.sr && sizeof(S) == 2) ? 1 : 0;
    a.step = s.d_step;
    a.nz = -0.0f;
    const float *K = stress ? s.Ks : s.Kv;
    const int nk = stress ? s.nks : s.nkv;
    for (int k = 0; k < OFD_MAX_K; ++k) a.K[k] = k < nk ? K[k] : 0.f;
    return a;
  }

  BcArgs<S> bc_args(const DevState &s, int t1, int t0, int recompute) const {
    BcArgs<S> a;
    a.g = s.g;
    for (int f = 0; f < NF; ++f) {
      a.f1[f] = fp(s, f, t1);
      a.f0[f] = fp(s, f, t0);
      a.sc[f] = s.scale[f];
      a.inv[f] = 1.f / s.scale[f];
    }
    for (int i = 0; i < NM; ++i) a.media[i] = s.media[i];
    for (int i = 0; i < 6; ++i) a.face[i] = s.face[i];
    a.recompute = recompute;
    a.dt = (C)s.dt;
    for (int i = 0; i < 3; ++i) a.h[i] = (C)s.h[i];
    a.c4[0] = (C)(9.0 / 8.0);
    a.c4[1] = (C)(-1.0 / 24.0);
    a.d = 0;
    a.sub = 0;
    a.gen = (R == 2 && sizeof(S) <= 4 && s.gen_ghost && s.d_kg) ? 1 : 0;
    a.het = s.het;
    a.kg = s.d_kg;
    a.rc = nullptr;
    a.rcs = s.rcs;
    return a;
  }

  static dim3 face_grid(const Geom &g, int d, int z) {
    int n1, n2;
    if (d == 0) { n1 = g.n2; n2 = g.n3; }
    else if (d == 1) { n1 = g.n1; n2 = g.n3; }
    else { n1 = g.n1; n2 = g.n2; }
    return dim3((n2 + 31) / 32, (n1 + 7) / 8, z);
  }

  // The step's generated recompute values (12 face planes).  rc_mode 1: on
  // the second stream after the work already queued on st (the previous
  // step's ghosts included), launched before the stress sweep at the highest
  // priority so that its blocks take the SM room the sweep's CTAs leave (its
  // FP64 work beside the memory-bound sweep); stress_bc waits for ev_join.
  // rc_mode 0: on st after the stress sweep.  The priority is a launch
  // attribute, so graph capture keeps it.
  static bool pre_ok(const DevState &s) {
    return R == 2 && sizeof(S) <= 4 && s.gen_ghost && s.d_kg && s.d_rc && s.st2 && !s.legacy;
  }
  void recompute_launch(const DevState &s, int t1, int t0, cudaStream_t st, int prio) {
    BcArgs<S> a = bc_args(s, t1, t0, 1);
    const Geom &g = s.g;
    const int nmax = std::max(g.n1, std::max(g.n2, g.n3));
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(sm_count() * std::max(1, s.rc_bps));
    cfg.blockDim = dim3(128);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributePriority;
    at[0].val.priority = prio;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, stress_recompute_kernel<R, S>, a, s.d_rc, nmax);
  }
  void pre_recompute(const DevState &s, int t1, int t0, cudaStream_t st) {
    cudaEventRecord(s.ev_fork, st);
    cudaStreamWaitEvent(s.st2, s.ev_fork, 0);
    recompute_launch(s, t1, t0, s.st2, greatest_priority());
    cudaEventRecord(s.ev_join, s.st2);
  }

  // pre: the recompute values are in d_rc (beside: computed on st2, so wait
  // for ev_join first)
  void stress_bc(const DevState &s, int t1, int t0, int recompute, cudaStream_t st, bool pre = false,
                 bool beside = false) {
    BcArgs<S> a = bc_args(s, t1, t0, recompute);
    if (pre) {
      if (beside) cudaStreamWaitEvent(st, s.ev_join, 0);
      a.rc = s.d_rc;
    }
    for (int d = 0; d < 3; ++d) {
      a.d = d;
      stress_bc_kernel<R, S><<<face_grid(s.g, d, 12), dim3(32, 8), 0, st>>>(a);
    }
  }

  // Velocity ghosts, one launch per face normal.  with_source: the first
  // launch also applies the source to the level-t1 stresses and advances the
  // device step counter (time stepping); boundary_init passes false.
  void velocity_bc(const DevState &s, int t1, bool with_source, cudaStream_t st) {
    BcArgs<S> a = bc_args(s, t1, t1, 0);
    for (int d = 0; d < 3; ++d) {
      a.d = d;
      if (a.gen)
        velocity_bc_gen_kernel<R, S><<<face_grid(s.g, d, 1), dim3(32, 8), 0, st>>>(
            a, fp(s, F_TXX, t1), fp(s, F_TYY, t1), fp(s, F_TZZ, t1), with_source ? s.src_off : -1L, s.d_wav, s.nt,
            with_source ? s.d_step : nullptr, s.scale[F_TXX], s.scale[F_TYY], s.scale[F_TZZ]);
      else
        velocity_bc_merged_kernel<R, S><<<face_grid(s.g, d, 1), dim3(32, 8), 0, st>>>(
            a, fp(s, F_TXX, t1), fp(s, F_TYY, t1), fp(s, F_TZZ, t1), with_source ? s.src_off : -1L, s.d_wav, s.nt,
            with_source ? s.d_step : nullptr, s.scale[F_TXX], s.scale[F_TYY], s.scale[F_TZZ]);
    }
  }

  void sweeps(const DevState &s, int t0, bool stress, cudaStream_t st) {
    SweepArgs<S> a = sweep_args(s, t0, stress);
    const Geom &g = s.g;
    const int nx = g.n1 - 2 * g.m, ny = g.n2 - 2 * g.m, nz = g.n3 - 2 * g.m;
    const int var = s.variant == 1 ? 1 : (stress ? s.var_stress : s.var_velocity);
    if (var != 1 && s.tiled.maps && tiled_supported<R, S>(g)) {
      if (s.het) {
        if (stress) launch_stress_tiled<R, S, 1>(a, s.tiled, t0, st);
        else launch_velocity_tiled<R, S, 1>(a, s.tiled, t0, st);
      } else {
        if (stress) launch_stress_tiled<R, S, 0>(a, s.tiled, t0, st);
        else launch_velocity_tiled<R, S, 0>(a, s.tiled, t0, st);
      }
      return;
    }
    // plain: aim for chunk_waves waves of 152 SMs x 8 CTAs
    const int bx = s.plain_bx > 0 ? s.plain_bx : 32, by = s.plain_by > 0 ? s.plain_by : 8;
    dim3 blk(bx, by);
    dim3 grd((nz + bx - 1) / bx, (ny + by - 1) / by, 1);
    long ctas = (long)grd.x * grd.y;
    const int waves = s.chunk_waves > 0 ? s.chunk_waves : 1;
    int chunks = (int)((152L * 8 * waves + ctas - 1) / ctas);
    if (chunks < 1) chunks = 1;
    if (chunks > nx) chunks = nx;
    a.xchunk = (nx + chunks - 1) / chunks;
    grd.z = (nx + a.xchunk - 1) / a.xchunk;
    if (s.het) {
      if (stress) stress_plain<R, S, 1><<<grd, blk, 0, st>>>(a);
      else velocity_plain<R, S, 1><<<grd, blk, 0, st>>>(a);
    } else {
      if (stress) stress_plain<R, S, 0><<<grd, blk, 0, st>>>(a);
      else velocity_plain<R, S, 0><<<grd, blk, 0, st>>>(a);
    }
  }

  // one trace row per completed step (row = device step counter - 1)
  void sample_receivers(const DevState &s, int t1, cudaStream_t st) {
    if (s.nrec <= 0) return;
    RecArgs<S> r = rec_args(s, t1);
    receiver_sample_kernel<S><<<(s.nrec + 127) / 128, 128, 0, st>>>(r);
  }

  RecArgs<S> rec_args(const DevState &s, int t1) const {
    RecArgs<S> r;
    for (int i = 0; i < 6; ++i) {
      const int f = i < 3 ? F_U + i : F_TXX + (i - 3);
      r.f[i] = fp(s, f, t1);
      r.inv[i] = 1.f / s.scale[f];
    }
    r.rec = s.d_rec;
    r.nrec = s.nrec;
    r.traces = s.d_traces;
    r.cap = s.rec_cap;
    r.step = s.d_step;
    return r;
  }

  void step(const DevState &s, int t0, cudaStream_t st, const StepEvents *ev) override {
    const int t1 = 1 - t0;
    auto rec = [&](int i) { if (ev) cudaEventRecord(ev->ev[i], st); };
    rec(0);
    const bool pre = pre_ok(s);
    const bool beside = pre && s.rc_mode == 1;
    if (beside) pre_recompute(s, t1, t0, st);
    sweeps(s, t0, true, st);
    rec(1);
    rec(2);
    if (pre && !beside) recompute_launch(s, t1, t0, st, 0);
    stress_bc(s, t1, t0, s.legacy ? 0 : 1, st, pre, beside);
    rec(3);
    rec(4);
    sweeps(s, t0, false, st);
    rec(5);
    rec(6);
    velocity_bc(s, t1, true, st);
    sample_receivers(s, t1, st);
    rec(7);
  }

  int launches_per_step(const DevState &s) const override {
    // 2 sweeps + 3 stress-ghost phases + 3 velocity-ghost phases (the first
    // carries the source and the step counter) + receivers, if any + the
    // precomputed normal-stress recompute of the generated ghosts, if any
    return 2 + 3 + 3 + (s.nrec > 0 ? 1 : 0) + (pre_ok(s) ? 1 : 0);
  }

  void boundary_init(const DevState &s, int level, cudaStream_t st) override {
    stress_bc(s, level, level, 0, st);
    velocity_bc(s, level, false, st);
  }

  void to_padded(const DevState &s, const float *dense, int f, int level, cudaStream_t st) override {
    dense_to_padded<S><<<1216, 256, 0, st>>>(dense, fp(s, f, level), s.g, s.scale[f]);
  }

  void from_padded(const DevState &s, float *dense, int f, int level, cudaStream_t st) override {
    padded_to_dense<S><<<1216, 256, 0, st>>>(fp(s, f, level), dense, s.g, 1.f / s.scale[f]);
  }

  void prepare(const DevState &s) override {
    if (s.het) {
      prepare_tiled<R, S, 1>();
    } else {
      prepare_tiled<R, S, 0>();
    }
  }

  int step_persistent(const DevState &s, int p0, int nsteps, cudaStream_t st) override {
    PersistArgs<S> a;
    for (int p = 0; p < 2; ++p) {
      a.st[p] = sweep_args(s, p, true);
      a.ve[p] = sweep_args(s, p, false);
      a.sbc[p] = bc_args(s, 1 - p, p, s.legacy ? 0 : 1);
      a.vbc[p] = bc_args(s, 1 - p, 1 - p, 0);
    }
    a.src_off = s.src_off;
    a.wav = s.d_wav;
    a.nt = s.nt;
    a.d_step = s.d_step;
    a.ssc[0] = s.scale[F_TXX];
    a.ssc[1] = s.scale[F_TYY];
    a.ssc[2] = s.scale[F_TZZ];
    a.bar = s.d_bar;
    a.err = s.tiled.err;
    a.wait_ns = s.tiled.wait_ns;
    for (int p = 0; p < 2; ++p) a.rec[p] = rec_args(s, 1 - p);
    a.nsteps = nsteps;
    a.p0 = p0;
    void *kern = s.het ? (void *)persistent_steps_kernel<R, S, 1> : (void *)persistent_steps_kernel<R, S, 0>;
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 256, 0);
    const Geom &g = s.g;
    const long npts = (long)(g.n1 - 2 * g.m) * (g.n2 - 2 * g.m) * (g.n3 - 2 * g.m);
    long want = (npts + 1023) / 1024;
    if (want < 16) want = 16;
    const long cap = (long)sms * (per_sm > 0 ? per_sm : 1);
    const unsigned blocks = (unsigned)(want < cap ? want : cap);
    void *args[] = {&a};
    // barrier words start from zero for every launch (an expired barrier of
    // an earlier launch may have left arrivals behind)
    cudaMemsetAsync(s.d_bar, 0, 2 * sizeof(unsigned), st);
    return (int)cudaLaunchCooperativeKernel(kern, dim3(blocks), dim3(256), args, 0, st);
  }

  // device tables of a group: sweeps [stress][t0], ghosts [t0]
  struct Plan : GroupPlanBase {
    cudaStream_t st = nullptr;
    int n = 0, het = 0;
    GroupSweep<S> *sw[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
    int sw_ctas[2][2] = {{0, 0}, {0, 0}};
    GroupBc<S> *sbc[2] = {nullptr, nullptr}, *vbc[2] = {nullptr, nullptr};
    int sbc_blocks[3] = {0, 0, 0}, vbc_blocks[3] = {0, 0, 0};
    bool kd[2] = {false, false};   // [stress]: literal tables follow KMap (register-held literals)
    bool receivers = false;        // some member records traces
    // generated-ghost recompute of the members that have it (rc_mode and
    // rc_bps as a single handle's)
    int rc_blocks = 0, rc_mode = 0, rc_bps = 16;
    cudaStream_t st2 = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
    std::vector<void *> raw;   // allocations (tables start 128-byte aligned inside them)
    // stream-ordered copy of a host table to a new 128-byte aligned device table
    template <typename T>
    cudaError_t upload(T **dst, const T *src, int count) {
      void *p = nullptr;
      cudaError_t e = cudaMallocAsync(&p, sizeof(T) * count + 128, st);
      if (e != cudaSuccess) return e;
      raw.push_back(p);
      *dst = (T *)(((uintptr_t)p + 127) & ~(uintptr_t)127);
      // pageable source: the copy is staged before the call returns
      return cudaMemcpyAsync(*dst, src, sizeof(T) * count, cudaMemcpyHostToDevice, st);
    }
    ~Plan() override {
      for (void *p : raw) cudaFreeAsync(p, st);
      if (st2) cudaStreamDestroy(st2);
      if (fork) cudaEventDestroy(fork);
      if (join) cudaEventDestroy(join);
    }
  };

  template <int HET, bool STRESS>
  cudaError_t build_sweep_table(const DevState *const *m, int n, int t0, int chunk_planes, Plan *pl) {
    std::vector<GroupSweep<S>> tab(n);
    std::vector<int> order(n), len(n);
    for (int i = 0; i < n; ++i) {
      tab[i].a = sweep_args(*m[i], t0, STRESS);
      int tiles, chunks;
      tiled_params<R, S, HET, STRESS>(tab[i].a, m[i]->tiled, t0, chunk_planes, tab[i].p, &tiles, &chunks);
      tab[i].tiles = tiles;
      tab[i].cta_begin = tiles * chunks;   // CTA count for now
      len[i] = tab[i].p.chunk;
      order[i] = i;
    }
    // longest CTAs first, so that the short ones fill the last wave
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return len[x] > len[y]; });
    std::vector<GroupSweep<S>> sorted(n);
    int total = 0;
    for (int i = 0; i < n; ++i) {
      sorted[i] = tab[order[i]];
      const int c = sorted[i].cta_begin;
      sorted[i].cta_begin = total;
      total += c;
    }
    pl->sw_ctas[STRESS ? 1 : 0][t0] = total;
    return pl->upload(&pl->sw[STRESS ? 1 : 0][t0], sorted.data(), n);
  }

  // Default x chunk of a group: the longest of 128, 112, ..., 16 planes that
  // still gives the whole launch ~8 waves of 152 SMs x 2 CTAs (long chunks
  // fetch fewer halo planes; enough CTAs keep every SM busy).
  static int group_chunk(const DevState *const *m, int n) {
    const long want = 152L * 2 * 8;
    for (int L = 128; L > 16; L -= 16) {
      long ctas = 0;
      for (int j = 0; j < n; ++j) {
        const Geom &g = m[j]->g;
        const long tiles = (long)((g.n3 - 2 * g.m + TZ - 1) / TZ) * ((g.n2 - 2 * g.m + tile_rows(R) - 1) / tile_rows(R));
        ctas += tiles * ((g.n1 - 2 * g.m + L - 1) / L);
      }
      if (ctas >= want) return L;
    }
    return 16;
  }

  // every member's table of this sweep repeats its values as KMap says
  template <bool STRESS>
  static bool tables_follow_kmap(const DevState *const *m, int n) {
    if constexpr (KMap<R, STRESS>::ok) {
      constexpr int NK = KMap<R, STRESS>::NK;
      for (int j = 0; j < n; ++j) {
        const float *K = STRESS ? m[j]->Ks : m[j]->Kv;
        if ((STRESS ? m[j]->nks : m[j]->nkv) != NK) return false;
        for (int i = 0; i < NK; ++i) {
          int f = 0;
          while (KMap<R, STRESS>::at(f) != KMap<R, STRESS>::at(i)) ++f;
          if (std::memcmp(&K[i], &K[f], sizeof(float)) != 0) return false;
        }
      }
      return true;
    }
    return false;
  }

  GroupPlanBase *group_build(const DevState *const *m, int n, int chunk_planes, cudaStream_t st,
                             cudaError_t *cuda_err) override {
    Plan *pl = new Plan();
    pl->st = st;
    pl->n = n;
    pl->het = m[0]->het;
    // groups run the recompute after the grouped stress sweep with a full
    // grid: measured faster than beside it for groups of 30-43 space-order-4
    // shots (128-192^3: 8.1 vs 10.6 s; 32-63^3: 0.97 vs 1.51 s)
    pl->rc_mode = 0;
    pl->rc_bps = 16;
    if (pl->het) {
      pl->kd[1] = tables_follow_kmap<true>(m, n);
      pl->kd[0] = tables_follow_kmap<false>(m, n);
    }
    if (chunk_planes <= 0) chunk_planes = group_chunk(m, n);
    cudaError_t e = cudaSuccess;
    for (int t0 = 0; t0 < 2 && e == cudaSuccess; ++t0) {
      if (pl->het) {
        e = build_sweep_table<1, true>(m, n, t0, chunk_planes, pl);
        if (e == cudaSuccess) e = build_sweep_table<1, false>(m, n, t0, chunk_planes, pl);
      } else {
        e = build_sweep_table<0, true>(m, n, t0, chunk_planes, pl);
        if (e == cudaSuccess) e = build_sweep_table<0, false>(m, n, t0, chunk_planes, pl);
      }
    }
    for (int t0 = 0; t0 < 2 && e == cudaSuccess; ++t0) {
      const int t1 = 1 - t0;
      std::vector<GroupBc<S>> stab(n), vtab(n);
      int sb[3] = {0, 0, 0}, vb[3] = {0, 0, 0};
      int rb = 0;
      for (int i = 0; i < n; ++i) {
        const DevState &s = *m[i];
        stab[i].a = bc_args(s, t1, t0, s.legacy ? 0 : 1);
        vtab[i].a = bc_args(s, t1, t1, 0);
        for (int d = 0; d < 3; ++d) {
          const dim3 fg = face_grid(s.g, d, 1);
          stab[i].bx[d] = vtab[i].bx[d] = (int)fg.x;
          stab[i].by[d] = vtab[i].by[d] = (int)fg.y;
          stab[i].begin[d] = sb[d];
          vtab[i].begin[d] = vb[d];
          sb[d] += (int)(fg.x * fg.y) * 12;
          vb[d] += (int)(fg.x * fg.y);
        }
        stab[i].step = nullptr;
        stab[i].src_off = -1;
        stab[i].a.rc = pre_ok(s) ? s.d_rc : nullptr;
        {
          const int nmax = std::max(s.g.n1, std::max(s.g.n2, s.g.n3));
          stab[i].rbx = vtab[i].rbx = (nmax + 31) / 32;
          stab[i].rby = vtab[i].rby = (nmax + 3) / 4;
          stab[i].rbegin = vtab[i].rbegin = rb;
          if (stab[i].a.rc) rb += stab[i].rbx * stab[i].rby * 12;
        }
        vtab[i].txx = fp(s, F_TXX, t1);
        vtab[i].tyy = fp(s, F_TYY, t1);
        vtab[i].tzz = fp(s, F_TZZ, t1);
        vtab[i].src_off = s.src_off;
        vtab[i].w = s.d_wav;
        vtab[i].nt = s.nt;
        vtab[i].step = s.d_step;
        vtab[i].s0 = s.scale[F_TXX];
        vtab[i].s1 = s.scale[F_TYY];
        vtab[i].s2 = s.scale[F_TZZ];
        vtab[i].rec = rec_args(s, t1);
        stab[i].rec = vtab[i].rec;
        if (s.nrec > 0) pl->receivers = true;
      }
      for (int d = 0; d < 3; ++d) {
        pl->sbc_blocks[d] = sb[d];
        pl->vbc_blocks[d] = vb[d];
      }
      pl->rc_blocks = rb;
      if (rb > 0 && !pl->st2) {
        if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&pl->st2, cudaStreamNonBlocking, greatest_priority());
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&pl->fork, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&pl->join, cudaEventDisableTiming);
      }
      e = pl->upload(&pl->sbc[t0], stab.data(), n);
      if (e == cudaSuccess) e = pl->upload(&pl->vbc[t0], vtab.data(), n);
    }
    if (e != cudaSuccess) {
      delete pl;
      *cuda_err = e;
      return nullptr;
    }
    return pl;
  }

  void group_step(GroupPlanBase *base, int t0, cudaStream_t st) override {
    Plan *pl = static_cast<Plan *>(base);
    const int n = pl->n;
    auto launch = [&](auto kern, int threads, int smem, int k) {
      kern<<<pl->sw_ctas[k][t0], threads, smem, st>>>(pl->sw[k][t0], n);
    };
    auto sweep = [&](bool stress) {
      const int k = stress ? 1 : 0;
      if (pl->het) {
        typedef TiledCfg<R, S, 1, true> GS;
        typedef TiledCfg<R, S, 1, false> GV;
        if (stress && pl->kd[1]) launch(sweep_tiled_group<R, S, 1, true, true>, GS::THREADS, GS::SMEM, k);
        else if (stress) launch(sweep_tiled_group<R, S, 1, true, false>, GS::THREADS, GS::SMEM, k);
        else if (pl->kd[0]) launch(sweep_tiled_group<R, S, 1, false, true>, GV::THREADS, GV::SMEM, k);
        else launch(sweep_tiled_group<R, S, 1, false, false>, GV::THREADS, GV::SMEM, k);
      } else {
        typedef TiledCfg<R, S, 0, true> GS;
        typedef TiledCfg<R, S, 0, false> GV;
        if (stress) launch(sweep_tiled_group<R, S, 0, true, false>, GS::THREADS, GS::SMEM, k);
        else launch(sweep_tiled_group<R, S, 0, false, false>, GV::THREADS, GV::SMEM, k);
      }
    };
    const bool pre = pl->rc_blocks > 0 && pl->st2;
    const bool beside = pre && pl->rc_mode == 1;
    auto recompute = [&](cudaStream_t rs, int prio) {
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(std::min(pl->rc_blocks, sm_count() * pl->rc_bps));
      cfg.blockDim = dim3(32, 4);
      cfg.dynamicSmemBytes = 0;
      cfg.stream = rs;
      cudaLaunchAttribute at[1];
      at[0].id = cudaLaunchAttributePriority;
      at[0].val.priority = prio;
      cfg.attrs = at;
      cfg.numAttrs = 1;
      cudaLaunchKernelEx(&cfg, stress_recompute_group_kernel<R, S>, (const GroupBc<S> *)pl->sbc[t0], n,
                         pl->rc_blocks);
    };
    if (beside) {
      cudaEventRecord(pl->fork, st);
      cudaStreamWaitEvent(pl->st2, pl->fork, 0);
      recompute(pl->st2, greatest_priority());
      cudaEventRecord(pl->join, pl->st2);
    }
    sweep(true);
    if (beside) cudaStreamWaitEvent(st, pl->join, 0);
    else if (pre) recompute(st, 0);
    for (int d = 0; d < 3; ++d)
      stress_bc_group_kernel<R, S><<<pl->sbc_blocks[d], dim3(32, 8), 0, st>>>(pl->sbc[t0], n, d);
    sweep(false);
    for (int d = 0; d < 3; ++d)
      velocity_bc_group_kernel<R, S><<<pl->vbc_blocks[d], dim3(32, 8), 0, st>>>(pl->vbc[t0], n, d);
    if (pl->receivers) receiver_sample_group_kernel<S><<<n, 128, 0, st>>>(pl->vbc[t0]);
  }

  bool tiled_ok(const DevState &s) const override { return s.tiled.maps && tiled_supported<R, S>(s.g); }

  bool kmap_ok(const DevState &s, bool stress) const override {
    const DevState *m[1] = {&s};
    return stress ? tables_follow_kmap<true>(m, 1) : tables_follow_kmap<false>(m, 1);
  }

  int ghost_table_size(int het) const override {
    if constexpr (R == 2 && sizeof(S) <= 4) return het ? GenGhost4<1>::NK : GenGhost4<0>::NK;
    return 0;
  }

  int table_size(int het, int stress) const override {
    if (het) return stress ? GenSweep<R, 1>::NK_STRESS : GenSweep<R, 1>::NK_VELOCITY;
    return stress ? GenSweep<R, 0>::NK_STRESS : GenSweep<R, 0>::NK_VELOCITY;
  }

  void absmax(const DevState &s, int level, double *d_out9, cudaStream_t st) override {
    const int nblk = 128;
    absmax_partial<S><<<dim3(nblk, NF), 256, 0, st>>>(s, level, s.d_partial);
    absmax_final<<<1, 32, 0, st>>>(s.d_partial, nblk, d_out9);
  }

  void sumsq(const DevState &s, int level, double *d_out9, cudaStream_t st) override {
    const int nblk = 128;
    sumsq_partial<S><<<dim3(nblk, NF), 256, 0, st>>>(s, level, s.d_partial);
    sumsq_final<<<1, 32, 0, st>>>(s.d_partial, nblk, d_out9);
  }
};

// Defines make_backend<S, OFD_INST_R> in an ofd_inst_<storage>.cu unit.
#define OFD_DEFINE_BACKEND(S) \
  template <> Backend *make_backend<S, OFD_INST_R>() { return new Impl<OFD_INST_R, S>(); }

}  // namespace ofd
