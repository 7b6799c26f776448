// Plain stress and velocity sweeps: one thread per (y, z) column, marching
// along x over a chunk of planes; neighbours come straight from global memory
// (L1/L2).  These are the correctness baseline and the fallback for shapes
// the tiled kernels do not cover.
//
// The arithmetic is the generated expression of csrc/generated/sweeps_gen.cuh
// (the reference generator's expanded, constant-folded C expression with its
// literals in a run-time table).  Mathematically (c_k the staggered weights of
// util.py:195-236):
//   D-_a f(i) = sum_k c_k (f[i+k-1] - f[i-k]) / h_a   (f staggered +1/2 on a)
//   D+_a f(i) = sum_k c_k (f[i+k]   - f[i-k+1]) / h_a (result staggered +1/2)
//   Txx' = (lam+2mu) D-_x U + lam (D-_y V + D-_z W), Tyy', Tzz' alike
//   Txy' = mu12 (D+_y U + D+_x V), Tyz' = mu23 (D+_z V + D+_y W),
//   Txz' = mu13 (D+_z U + D+_x W)
//   U' = beta1 (D+_x Txx + D-_y Txy + D-_z Txz)
//   V' = beta2 (D-_x Txy + D+_y Tyy + D-_z Tyz)
//   W' = beta3 (D-_x Txz + D-_y Tyz + D+_z Tzz)
#pragma once
#include "ofd_common.cuh"
#include "generated/sweeps_gen.cuh"

namespace ofd {

// Accessor of the generated update expressions for the plain kernels:
// A(f, dx, dy, dz) loads field f at offset (dx, dy, dz) from the current
// point, A.m(i) the media array i at the point.
template <typename S>
struct PlainAcc {
  typedef typename Storage<S>::C C;
  const SweepArgs<S> &a;
  long o;
  __device__ __forceinline__ C operator()(int f, int dx, int dy, int dz) const {
    return (C)Storage<S>::load(a.in[f][o + dx * a.g.plane + dy * a.g.P + dz], a.inv[f]);
  }
  __device__ __forceinline__ C m(int i) const { return (C)a.media[i][o]; }
};

template <int R, typename S, int HET>
__global__ void __launch_bounds__(256) stress_plain(const __grid_constant__ SweepArgs<S> a) {
  typedef typename Storage<S>::C C;
  const Geom &g = a.g;
  const int z = g.m + blockIdx.x * blockDim.x + threadIdx.x;
  const int y = g.m + blockIdx.y * blockDim.y + threadIdx.y;
  if (z >= g.n3 - g.m || y >= g.n2 - g.m) return;
  const int xb = g.m + blockIdx.z * a.xchunk;
  const int xe = min(xb + a.xchunk, g.n1 - g.m);
  const long step = a.sr ? *a.step : 0;
  for (int x = xb; x < xe; ++x) {
    const long o = (long)x * g.plane + (long)y * g.P + z;
    PlainAcc<S> A{a, o};
    C out[6];
    GenSweep<R, HET>::template stress<C>(A, (const float *)a.K, out);
#pragma unroll
    for (int i = 0; i < 6; ++i)
      a.out[F_TXX + i][o] = SweepStore<S>::st(out[i], a.sc[F_TXX + i], a.sr, a.sr ? sr_hash(o, F_TXX + i, step) : 0u);
  }
}

template <int R, typename S, int HET>
__global__ void __launch_bounds__(256) velocity_plain(const __grid_constant__ SweepArgs<S> a) {
  typedef typename Storage<S>::C C;
  const Geom &g = a.g;
  const int z = g.m + blockIdx.x * blockDim.x + threadIdx.x;
  const int y = g.m + blockIdx.y * blockDim.y + threadIdx.y;
  if (z >= g.n3 - g.m || y >= g.n2 - g.m) return;
  const int xb = g.m + blockIdx.z * a.xchunk;
  const int xe = min(xb + a.xchunk, g.n1 - g.m);
  const long step = a.sr ? *a.step : 0;
  for (int x = xb; x < xe; ++x) {
    const long o = (long)x * g.plane + (long)y * g.P + z;
    PlainAcc<S> A{a, o};
    C out[3];
    GenSweep<R, HET>::template velocity<C>(A, (const float *)a.K, out);
#pragma unroll
    for (int i = 0; i < 3; ++i)
      a.out[F_U + i][o] = SweepStore<S>::st(out[i], a.sc[F_U + i], a.sr, a.sr ? sr_hash(o, F_U + i, step) : 0u);
  }
}

}  // namespace ofd
