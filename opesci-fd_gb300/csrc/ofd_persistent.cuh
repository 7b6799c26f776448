// Persistent time stepping for small grids: one cooperative launch advances
// a simulation many steps.  Every phase of a step (stress sweep, three stress
// ghost phases, velocity sweep, three velocity ghost phases with the source)
// is a grid-stride loop over the whole grid, separated by a grid barrier, so
// a step costs 8 barriers instead of 8 kernel launches.  Small grids, whose
// steps are shorter than a few kernel launches, are the ones that gain.
//
// The barrier is this library's own: a counter and a generation word in
// device memory, waited on with a wall-time bound (10 s) after which the
// block records an error and leaves.  Cooperative launch guarantees that all
// blocks are resident, so the barrier cannot wait on a block that never
// runs.  Reads of field values go through L2 only (ld.global.cg): another
// block wrote them earlier in this launch and this SM's L1 may hold an older
// copy of the line.
#pragma once
#include "ofd_common.cuh"
#include "ofd_bc.cuh"
#include "generated/sweeps_gen.cuh"

namespace ofd {

template <typename S>
struct CoherentAcc {
  typedef typename Storage<S>::C C;
  const SweepArgs<S> &a;
  long o;
  __device__ __forceinline__ C operator()(int f, int dx, int dy, int dz) const {
    return (C)Storage<S>::load(__ldcg(&a.in[f][o + dx * a.g.plane + dy * a.g.P + dz]), a.inv[f]);
  }
  __device__ __forceinline__ C m(int i) const { return (C)a.media[i][o]; }
};

template <typename S>
struct PersistArgs {
  SweepArgs<S> st[2];   // stress sweep by parity of t0
  SweepArgs<S> ve[2];   // velocity sweep by parity of t0
  BcArgs<S> sbc[2];     // stress ghosts (level t1, recompute reads t0)
  BcArgs<S> vbc[2];     // velocity ghosts (level t1)
  long src_off;         // -1: no source
  const float *wav;
  int nt;
  long *d_step;
  float ssc[3];         // storage scales of Txx Tyy Tzz
  unsigned *bar;        // [0] arrivals, [1] generation
  int *err;
  unsigned long long wait_ns;   // limit of each grid-barrier wait (handle setting)
  int nsteps;
  int p0;               // parity of the first step
  RecArgs<S> rec[2];    // receivers by parity of t0 (level t1 = 1 - p)
};

__device__ __forceinline__ unsigned long long wall_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}

// Bounded grid barrier; false when its wait (limit_ns of %globaltimer) or
// another block's expired.  A waiting block also leaves as soon as another
// block has set the error word, so one expiry ends every block's wait.
__device__ __forceinline__ bool grid_barrier(unsigned *bar, int *err, unsigned long long limit_ns) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned *gen = bar + 1;
    const unsigned g = *gen;
    __threadfence();
    const unsigned nb = gridDim.x;
    int ok = 1;
    if (atomicAdd(bar, 1u) == nb - 1) {
      atomicExch(bar, 0u);
      __threadfence();
      atomicAdd(bar + 1, 1u);
    } else {
      const unsigned long long t0 = wall_ns();
      while (*gen == g) {
        __nanosleep(32);
        if (*(volatile int *)err) {
          ok = 0;
          break;
        }
        if (wall_ns() - t0 > limit_ns) {
          atomicExch(err, 3);
          ok = 0;
          break;
        }
      }
    }
    __threadfence();
    if (*(volatile int *)err) ok = 0;
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

template <int R, typename S, int HET>
__global__ void __launch_bounds__(256) persistent_steps_kernel(const __grid_constant__ PersistArgs<S> a) {
  typedef typename Storage<S>::C C;
  const Geom &g = a.st[0].g;
  const long gtid = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const long gstride = (long)gridDim.x * blockDim.x;
  const int nx = g.n1 - 2 * g.m, ny = g.n2 - 2 * g.m, nz = g.n3 - 2 * g.m;
  const long npts = (long)nx * ny * nz;
  // the step count before this launch (read by every block before the first
  // grid barrier; block 0 advances the counter only after it)
  const long step0 = *(volatile long *)a.d_step;
  for (int k = 0; k < a.nsteps; ++k) {
    const int p = (a.p0 + k) & 1;
    const long step = step0 + k;
    // stress sweep
    {
      const SweepArgs<S> &sa = a.st[p];
      for (long i = gtid; i < npts; i += gstride) {
        const int z = g.m + (int)(i % nz);
        const long r = i / nz;
        const int y = g.m + (int)(r % ny);
        const int x = g.m + (int)(r / ny);
        const long o = (long)x * g.plane + (long)y * g.P + z;
        CoherentAcc<S> A{sa, o};
        C out[6];
        GenSweep<R, HET>::template stress<C>(A, (const float *)sa.K, out);
#pragma unroll
        for (int f = 0; f < 6; ++f)
          sa.out[F_TXX + f][o] =
              SweepStore<S>::st(out[f], sa.sc[F_TXX + f], sa.sr, sa.sr ? sr_hash(o, F_TXX + f, step) : 0u);
      }
    }
    if (!grid_barrier(a.bar, a.err, a.wait_ns)) return;
    // stress ghosts, one phase per face normal
    for (int d = 0; d < 3; ++d) {
      int a1, a2;
      plane_axes(d, a1, a2);
      const int n1 = gdim(g, a1), n2 = gdim(g, a2);
      const long nitems = (long)n1 * n2 * 12;
      for (long i = gtid; i < nitems; i += gstride) {
        const int i2 = (int)(i % n2);
        const long r = i / n2;
        const int i1 = (int)(r % n1);
        const int zz = (int)(r / n1);
        stress_bc_point<R, S, true>(a.sbc[p], d, i1, i2, zz >> 1, zz & 1);
      }
      if (!grid_barrier(a.bar, a.err, a.wait_ns)) return;
    }
    // velocity sweep
    {
      const SweepArgs<S> &va = a.ve[p];
      for (long i = gtid; i < npts; i += gstride) {
        const int z = g.m + (int)(i % nz);
        const long r = i / nz;
        const int y = g.m + (int)(r % ny);
        const int x = g.m + (int)(r / ny);
        const long o = (long)x * g.plane + (long)y * g.P + z;
        CoherentAcc<S> A{va, o};
        C out[3];
        GenSweep<R, HET>::template velocity<C>(A, (const float *)va.K, out);
#pragma unroll
        for (int f = 0; f < 3; ++f)
          va.out[F_U + f][o] = SweepStore<S>::st(out[f], va.sc[F_U + f], va.sr, va.sr ? sr_hash(o, F_U + f, step) : 0u);
      }
    }
    if (!grid_barrier(a.bar, a.err, a.wait_ns)) return;
    // velocity ghosts, one phase per face normal; the source and the step
    // counter ride on the first
    for (int d = 0; d < 3; ++d) {
      int a1, a2;
      plane_axes(d, a1, a2);
      const int n1 = gdim(g, a1), n2 = gdim(g, a2);
      const long nitems = (long)n1 * n2;
      for (long i = gtid; i < nitems; i += gstride) {
        velocity_bc_merged_point<R, S, true>(a.vbc[p], d, (int)(i / n2), (int)(i % n2));
      }
      if (d == 0 && gtid == 0) {
        const long st = *(volatile long *)a.d_step;
        if (a.src_off >= 0 && st < a.nt) {
          S *t[3] = {a.st[p].out[F_TXX], a.st[p].out[F_TYY], a.st[p].out[F_TZZ]};
#pragma unroll
          for (int q = 0; q < 3; ++q) {
            const float v = a.wav[(long)q * a.nt + st] / 3;   // x, y, z signals
            const C old = Storage<S>::load(__ldcg(&t[q][a.src_off]), 1.f / a.ssc[q]);
            t[q][a.src_off] = Storage<S>::store(old - v, a.ssc[q]);
          }
        }
        *a.d_step = st + 1;
      }
      if (!grid_barrier(a.bar, a.err, a.wait_ns)) return;
    }
    // receivers read level t1, which the next step's phases do not write
    // (they write the other level), so no barrier follows
    const RecArgs<S> &rc = a.rec[p];
    if (rc.nrec > 0) {
      const long row = *(volatile long *)a.d_step - 1;
      if (row >= 0 && row < rc.cap)
        for (long i = gtid; i < rc.nrec; i += gstride) sample_receiver_coherent(rc, row, (int)i);
    }
  }
}

}  // namespace ofd
