// Plain stress and velocity sweeps: one thread per (y, z) column, marching
// along x over a chunk of planes; neighbours come straight from global memory
// (L1/L2).  These are the correctness baseline and the fallback for shapes
// the tiled kernels do not cover.
//
// Update formulas (the expanded kernels of staggeredgrid.py:728-748 regrouped
// as weighted differences, c_k the staggered weights of util.py:195-236):
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

namespace ofd {

template <int R, typename S>
__global__ void __launch_bounds__(256) stress_plain(SweepArgs<S> a) {
  typedef typename Storage<S>::C C;
  const Geom g = a.g;
  const int z = g.m + blockIdx.x * blockDim.x + threadIdx.x;
  const int y = g.m + blockIdx.y * blockDim.y + threadIdx.y;
  if (z >= g.n3 - g.m || y >= g.n2 - g.m) return;
  const int xb = g.m + blockIdx.z * a.xchunk;
  const int xe = min(xb + a.xchunk, g.n1 - g.m);
  const long sx = g.plane, sy = g.P;
  for (int x = xb; x < xe; ++x) {
    const long o = x * sx + y * sy + z;
    auto L = [&](int f, long off) -> C { return (C)Storage<S>::load(a.in[f][o + off], a.inv[f]); };
    C dxU = 0, dyV = 0, dzW = 0, dyU = 0, dxV = 0, dzV = 0, dyW = 0, dzU = 0, dxW = 0;
#pragma unroll
    for (int k = 1; k <= R; ++k) {
      const C c = a.c[k - 1];
      dxU += c * (L(F_U, (k - 1) * sx) - L(F_U, -k * sx));
      dyV += c * (L(F_V, (k - 1) * sy) - L(F_V, -k * sy));
      dzW += c * (L(F_W, (k - 1)) - L(F_W, -k));
      dyU += c * (L(F_U, k * sy) - L(F_U, (1 - k) * sy));
      dxV += c * (L(F_V, k * sx) - L(F_V, (1 - k) * sx));
      dzV += c * (L(F_V, k) - L(F_V, (1 - k)));
      dyW += c * (L(F_W, k * sy) - L(F_W, (1 - k) * sy));
      dzU += c * (L(F_U, k) - L(F_U, (1 - k)));
      dxW += c * (L(F_W, k * sx) - L(F_W, (1 - k) * sx));
    }
    dxU *= a.ih1; dxV *= a.ih1; dxW *= a.ih1;
    dyU *= a.ih2; dyV *= a.ih2; dyW *= a.ih2;
    dzU *= a.ih3; dzV *= a.ih3; dzW *= a.ih3;
    const long mo = (long)x * g.plane + (long)y * g.P + z;
    const C lam = (C)a.media[M_LAM][mo], mu = (C)a.media[M_MU][mo];
    const C l2m = lam + C(2) * mu;
    const C dt = a.dt;
    a.out[F_TXX][o] = Storage<S>::store(L(F_TXX, 0) + dt * (l2m * dxU + lam * (dyV + dzW)), a.sc[F_TXX]);
    a.out[F_TYY][o] = Storage<S>::store(L(F_TYY, 0) + dt * (l2m * dyV + lam * (dxU + dzW)), a.sc[F_TYY]);
    a.out[F_TZZ][o] = Storage<S>::store(L(F_TZZ, 0) + dt * (l2m * dzW + lam * (dxU + dyV)), a.sc[F_TZZ]);
    a.out[F_TXY][o] = Storage<S>::store(L(F_TXY, 0) + dt * ((C)a.media[M_MU12][mo] * (dyU + dxV)), a.sc[F_TXY]);
    a.out[F_TYZ][o] = Storage<S>::store(L(F_TYZ, 0) + dt * ((C)a.media[M_MU23][mo] * (dzV + dyW)), a.sc[F_TYZ]);
    a.out[F_TXZ][o] = Storage<S>::store(L(F_TXZ, 0) + dt * ((C)a.media[M_MU13][mo] * (dzU + dxW)), a.sc[F_TXZ]);
  }
}

template <int R, typename S>
__global__ void __launch_bounds__(256) velocity_plain(SweepArgs<S> a) {
  typedef typename Storage<S>::C C;
  const Geom g = a.g;
  const int z = g.m + blockIdx.x * blockDim.x + threadIdx.x;
  const int y = g.m + blockIdx.y * blockDim.y + threadIdx.y;
  if (z >= g.n3 - g.m || y >= g.n2 - g.m) return;
  const int xb = g.m + blockIdx.z * a.xchunk;
  const int xe = min(xb + a.xchunk, g.n1 - g.m);
  const long sx = g.plane, sy = g.P;
  for (int x = xb; x < xe; ++x) {
    const long o = x * sx + y * sy + z;
    auto L = [&](int f, long off) -> C { return (C)Storage<S>::load(a.in[f][o + off], a.inv[f]); };
    C u = 0, v = 0, w = 0;
#pragma unroll
    for (int k = 1; k <= R; ++k) {
      const C c = a.c[k - 1];
      // U: D+x Txx, D-y Txy, D-z Txz
      u += c * ((L(F_TXX, k * sx) - L(F_TXX, (1 - k) * sx)) * a.ih1 +
                (L(F_TXY, (k - 1) * sy) - L(F_TXY, -k * sy)) * a.ih2 +
                (L(F_TXZ, (k - 1)) - L(F_TXZ, -k)) * a.ih3);
      // V: D-x Txy, D+y Tyy, D-z Tyz
      v += c * ((L(F_TXY, (k - 1) * sx) - L(F_TXY, -k * sx)) * a.ih1 +
                (L(F_TYY, k * sy) - L(F_TYY, (1 - k) * sy)) * a.ih2 +
                (L(F_TYZ, (k - 1)) - L(F_TYZ, -k)) * a.ih3);
      // W: D-x Txz, D-y Tyz, D+z Tzz
      w += c * ((L(F_TXZ, (k - 1) * sx) - L(F_TXZ, -k * sx)) * a.ih1 +
                (L(F_TYZ, (k - 1) * sy) - L(F_TYZ, -k * sy)) * a.ih2 +
                (L(F_TZZ, k) - L(F_TZZ, (1 - k))) * a.ih3);
    }
    const long mo = (long)x * g.plane + (long)y * g.P + z;
    const C dt = a.dt;
    a.out[F_U][o] = Storage<S>::store(L(F_U, 0) + dt * ((C)a.media[M_B1][mo] * u), a.sc[F_U]);
    a.out[F_V][o] = Storage<S>::store(L(F_V, 0) + dt * ((C)a.media[M_B2][mo] * v), a.sc[F_V]);
    a.out[F_W][o] = Storage<S>::store(L(F_W, 0) + dt * ((C)a.media[M_B3][mo] * w), a.sc[F_W]);
  }
}

}  // namespace ofd
