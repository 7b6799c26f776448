// Free-surface ghost cells (stress and velocity), restating the ghost
// equations of fields.py:192-381 and the loop ranges/order of
// staggeredgrid.py:754-864.
//
// Phases.  The reference updates ghosts field by field, face normal by face
// normal (x, then y, then z), and later faces read values written by earlier
// ones (corners, and the Levander recompute overwriting planes a mirror has
// read).  One launch per face normal d reproduces that: within a phase the
// fields and the two sides are independent.  Velocity ghosts of one normal
// are ordered too: the component along d first (staggeredgrid.py:829-832),
// then the two tangential components that read it at their point and at the
// next point along their own axis; the kernel below recomputes that
// neighbour's value instead of reading it, so one launch per normal suffices.
//
// Stress, face normal d, plane index b (lower b = m, upper b = n-m-1):
//  * normal stress T_dd (unstaggered along d): T[b] = 0, T[b-+k] = -T[b+-k],
//    k = 1..R-1; in-plane range [0, n) (fields.py:361-381);
//  * shear stress with d among its indices (staggered along d):
//    lower T[b-1-k] = -T[b+k], upper T[b+k] = -T[b-1-k], k = 0..R-1;
//  * Levander, normal stress T_aa with a != d, plane b, in-plane range
//    [m+1, n-m-1): T_aa(t1) = T_aa(t0) + dt (K1 D4_a v_a + K2 D4_e v_e) with
//    K1 = lam+2mu - lam^2/(lam+2mu), K2 = lam - lam^2/(lam+2mu): the rate of
//    T_aa with dv_d/dx_d eliminated through T_dd = 0 (fields.py:313-353).
// Velocity, face normal d, in-plane range [1, n-1):
//  * Levander, component along d (zero normal traction, 2nd-order FD):
//    lower v_d[b-1] = v_d[b] + r sum_j (h_d/h_j)(v_j[b; j] - v_j[b; j-1]),
//    upper v_d[b]   = v_d[b-1] - r sum_j (h_d/h_j)(v_j[b; j] - v_j[b; j-1]),
//    r = lam/(lam+2mu) at plane b (fields.py:220-224);
//  * Levander, tangential v_j (continuity of dT_jd/dt across the surface,
//    fields.py:225-230), with G(p) = h_d (v_d[p; j+1] - v_d[p; j]) / h_j and
//    mu_lo, mu_hi the effective shear modulus of T_jd at planes b-1, b:
//    lower v_j[b-1] = v_j[b] + G(b-1) - (mu_hi/mu_lo)(v_j[b+1] - v_j[b] + G(b)),
//    upper v_j[b+1] = v_j[b] - G(b) + (mu_lo/mu_hi)(v_j[b] - v_j[b-1] + G(b-1));
//  * Robertsson: R ghost layers set to zero (fields.py:243-259).
//
// Space order 4 with the generated ghost expressions (BcArgs::gen): the
// recomputed normal stresses and the Levander velocity ghosts are the
// frontend's own printed ghost equations (generated/ghosts_gen.cuh), term for
// term, which makes the ghost values bit for bit those of the reference's C.
// The formulas above stay as the path for FP64 storage and for models whose
// ghost equations have another structure.
#pragma once
#include "ofd_common.cuh"
#include "generated/ghosts_gen.cuh"

namespace ofd {

// Global loads of field values: COH = true reads through L2 only
// (ld.global.cg), which a kernel needs when it reads values that other CTAs
// wrote earlier in the same launch (the persistent step kernel).
template <bool COH, typename S>
__device__ __forceinline__ S ldg(const S *p) {
  if (COH) return __ldcg(p);
  return *p;
}

__device__ __forceinline__ void plane_axes(int d, int &a1, int &a2) {
  // a2 is the faster-varying in-plane axis (mapped to threadIdx.x)
  if (d == 0) { a1 = 1; a2 = 2; }
  else if (d == 1) { a1 = 0; a2 = 2; }
  else { a1 = 0; a2 = 1; }
}

__device__ __forceinline__ long lin(const Geom &g, int x, int y, int z) {
  return (long)x * g.plane + (long)y * g.P + z;
}

// offset of the point with in-plane coordinates (p1, p2) (axes of
// plane_axes(d)) and coordinate pd along d; no runtime-indexed arrays, so
// nothing lands in local memory
__device__ __forceinline__ long plane_lin(const Geom &g, int d, int p1, int p2, int pd) {
  if (d == 0) return lin(g, pd, p1, p2);
  if (d == 1) return lin(g, p1, pd, p2);
  return lin(g, p1, p2, pd);
}

__device__ __forceinline__ int gdim(const Geom &g, int a) { return a == 0 ? g.n1 : (a == 1 ? g.n2 : g.n3); }

// stride of axis a in elements
__device__ __forceinline__ long gstride(const Geom &g, int a) { return a == 0 ? g.plane : (a == 1 ? g.P : 1); }

__device__ __forceinline__ int mu_pair(int a, int b) {
  const int lo = a < b ? a : b, hi = a < b ? b : a;
  if (lo == 0 && hi == 1) return M_MU12;
  if (lo == 0 && hi == 2) return M_MU13;
  return M_MU23;
}

// Accessor of the generated ghost expressions: A(F, level, ox, oy, oz) is
// field F at level t0 (0) or t1 (1) at an offset from the point o on the
// boundary plane, A.m(M, ox, oy, oz) a medium there.  For the tangential
// velocity ghosts, the along-d component's ghost at this point (offset go)
// and at the next point along axis ja is the fresh value (v0, vn) the same
// launch computes, as the reference's face order has written it by then.
template <typename S, bool COH>
struct GhostAcc {
  const BcArgs<S> &a;
  long o;
  int fd;          // field whose fresh ghost values are used (-1: none)
  int gd, gv;      // that ghost sits at offset gv along axis gd from this point
  int ja;          // axis of the neighbour holding vn
  float v0, vn;
  __device__ __forceinline__ float operator()(int f, int lvl, int ox, int oy, int oz) const {
    if (f == fd) {
      const int ex = ox - (gd == 0 ? gv : 0), ey = oy - (gd == 1 ? gv : 0), ez = oz - (gd == 2 ? gv : 0);
      if (ex == 0 && ey == 0 && ez == 0) return v0;
      if (ex == (ja == 0) && ey == (ja == 1) && ez == (ja == 2)) return vn;
    }
    const S *p = lvl ? (const S *)a.f1[f] : a.f0[f];
    return (float)Storage<S>::load(ldg<COH>(&p[o + ox * a.g.plane + oy * a.g.P + oz]), a.inv[f]);
  }
  __device__ __forceinline__ float m(int i, int ox, int oy, int oz) const {
    return a.media[i][o + ox * a.g.plane + oy * a.g.P + oz];
  }
};

template <typename S, bool COH>
__device__ __forceinline__ GhostAcc<S, COH> ghost_acc(const BcArgs<S> &a, long o) {
  return GhostAcc<S, COH>{a, o, -1, 0, 0, 0, 0.f, 0.f};
}

// generated velocity ghost of component c on face (d, side) at point o of
// the boundary plane, through accessor A
template <class Acc, class S>
__device__ __forceinline__ float gen_velocity_ghost(const BcArgs<S> &a, int c, int d, int side, const Acc &A) {
  return a.het ? GenGhost4<1>::velocity(c, d, side, A, a.kg) : GenGhost4<0>::velocity(c, d, side, A, a.kg);
}

// generated normal-stress recompute value of stress fi on face (d, side)
template <class Acc, class S>
__device__ __forceinline__ float gen_stress_recompute(const BcArgs<S> &a, int fi, int d, int side, const Acc &A) {
  return a.het ? GenGhost4<1>::stress(fi, d, side, A, a.kg) : GenGhost4<0>::stress(fi, d, side, A, a.kg);
}

// Stress ghosts of face normal d at in-plane point (i1, i2) for stress
// component fi (0..5) and side.
template <int R, typename S, bool COH>
__device__ __forceinline__ void stress_bc_point(const BcArgs<S> &a, int d, int i1, int i2, int fi, int side) {
  typedef typename Storage<S>::C C;
  const Geom &g = a.g;
  int a1, a2;
  plane_axes(d, a1, a2);
  const int n1 = gdim(g, a1), n2 = gdim(g, a2), nd = gdim(g, d);
  if (i1 >= n1 || i2 >= n2) return;
  const int fb = a.face[2 * d + side];
  if (fb == 0) return;
  const int F = F_TXX + fi;
  // directions of the stress component
  const int dA = (fi < 3) ? fi : (fi == 3 ? 0 : (fi == 4 ? 1 : 0));
  const int dB = (fi < 3) ? fi : (fi == 3 ? 1 : 2);
  const bool normal = fi < 3;
  const int m = g.m;
  const int b = side == 0 ? m : nd - m - 1;
  const long base = plane_lin(g, d, i1, i2, 0);
  const long sd = gstride(g, d);
  S *T = a.f1[F];
  if (d == dA || d == dB) {
    if (normal) {
      T[base + b * sd] = Storage<S>::store(C(0), a.sc[F]);
      const int sgn = side == 0 ? -1 : 1;
#pragma unroll
      for (int k = 1; k < R; ++k) {
        const C v = Storage<S>::load(ldg<COH>(&T[base + (b - sgn * k) * sd]), a.inv[F]);
        T[base + (b + sgn * k) * sd] = Storage<S>::store(-v, a.sc[F]);
      }
    } else {
#pragma unroll
      for (int k = 0; k < R; ++k) {
        const int dst = side == 0 ? b - 1 - k : b + k;
        const int src = side == 0 ? b + k : b - 1 - k;
        const C v = Storage<S>::load(ldg<COH>(&T[base + src * sd]), a.inv[F]);
        T[base + dst * sd] = Storage<S>::store(-v, a.sc[F]);
      }
    }
    return;
  }
  if (!normal || fb != 1 || !a.recompute) return;
  if (i1 < m + 1 || i1 >= n1 - m - 1 || i2 < m + 1 || i2 >= n2 - m - 1) return;
  // Levander recompute of T_aa (a = dA) on plane b
  if constexpr (R == 2 && sizeof(S) <= 4) {
    if (a.gen) {
      const long o = base + b * sd;
      float v;
      if (a.rc) {
        const int q = fi > d ? fi - 1 : fi;
        v = a.rc[((d * 2 + side) * 2 + q) * a.rcs + (long)i1 * n2 + i2];
      } else {
        const auto A = ghost_acc<S, COH>(a, o);
        v = gen_stress_recompute(a, fi, d, side, A);
      }
      T[o] = Storage<S>::store(v, a.sc[F]);
      return;
    }
  }
  const int ax = dA;
  const int e = 3 - ax - d;
  const long o = base + b * sd;
  const C lam = (C)a.media[M_LAM][o], mu = (C)a.media[M_MU][o];
  const C l2m = lam + C(2) * mu;
  const C q = lam * lam / l2m;
  const C K1 = l2m - q, K2 = lam - q;
  const long sa = gstride(g, ax), se = gstride(g, e);
  const S *va = a.f0[F_U + ax], *ve = a.f0[F_U + e];
  auto LV = [&](const S *p, int f, long off) -> C { return Storage<S>::load(ldg<COH>(&p[o + off]), a.inv[f]); };
  const C Da = (a.c4[0] * (LV(va, F_U + ax, 0) - LV(va, F_U + ax, -sa)) +
                a.c4[1] * (LV(va, F_U + ax, sa) - LV(va, F_U + ax, -2 * sa))) / a.h[ax];
  const C De = (a.c4[0] * (LV(ve, F_U + e, 0) - LV(ve, F_U + e, -se)) +
                a.c4[1] * (LV(ve, F_U + e, se) - LV(ve, F_U + e, -2 * se))) / a.h[e];
  const C t0 = Storage<S>::load(ldg<COH>(&a.f0[F][o]), a.inv[F]);
  T[o] = Storage<S>::store(t0 + a.dt * (K1 * Da + K2 * De), a.sc[F]);
}

// The generated normal-stress recompute values of one step, all face normals
// at once, into rc (layout of BcArgs::rc).  Its inputs are the level-t0
// stresses and velocities and the media, all final before the step starts,
// so the runtime may run it on a second stream beside the stress sweep; the
// FP64 terms of the heterogeneous expressions (pow(mu, 2) makes the rest of
// each sum double) then use the FP64 units the memory-bound sweep leaves
// idle.  Grid-stride over virtual 32 x 4 tiles of the 12 face planes (lane:
// i2, warp: i1), so that a small grid of a few blocks per SM covers it.
// At most 40 registers a thread: two space-order-4 sweep CTAs (288 threads
// x 96 registers each) leave 10,240 registers of an SM, room for two such
// blocks beside them.
template <int R, typename S>
__global__ void __launch_bounds__(128, 12) stress_recompute_kernel(const __grid_constant__ BcArgs<S> a, float *rc, int nmax) {
  if constexpr (R == 2 && sizeof(S) <= 4) {
    const Geom &g = a.g;
    const int m = g.m;
    const int tx = (nmax + 31) >> 5, ty = (nmax + 3) >> 2;
    const int per = tx * ty;
    for (int vb = blockIdx.x; vb < 12 * per; vb += gridDim.x) {
      const int z = vb / per;
      const int r = vb - z * per;
      const int i1 = (r / tx) * 4 + (int)(threadIdx.x >> 5);
      const int i2 = (r % tx) * 32 + (int)(threadIdx.x & 31);
      const int q = z & 1, side = (z >> 1) & 1, d = z >> 2;
      int a1, a2;
      plane_axes(d, a1, a2);
      const int n1 = gdim(g, a1), n2 = gdim(g, a2), nd = gdim(g, d);
      if (i1 < m + 1 || i1 >= n1 - m - 1 || i2 < m + 1 || i2 >= n2 - m - 1) continue;
      if (a.face[2 * d + side] != 1) continue;
      const int fi = q < d ? q : q + 1;
      const int b = side == 0 ? m : nd - m - 1;
      const auto A = ghost_acc<S, false>(a, plane_lin(g, d, i1, i2, b));
      const float v =
          gen_stress_recompute(a, fi, d, side, A);
      rc[(long)z * a.rcs + (long)i1 * n2 + i2] = v;
    }
  }
}

// Stress ghosts of face normal a.d: blockIdx.z = field(0..5)*2 + side.
template <int R, typename S>
__global__ void __launch_bounds__(256) stress_bc_kernel(const __grid_constant__ BcArgs<S> a) {
  const int i2 = blockIdx.x * blockDim.x + threadIdx.x;
  const int i1 = blockIdx.y * blockDim.y + threadIdx.y;
  stress_bc_point<R, S, false>(a, a.d, i1, i2, blockIdx.z >> 1, blockIdx.z & 1);
}

// Velocity ghosts of face normal d at in-plane point (i1, i2).  sub 0: the
// component along d, zi = side; sub 1: zi = which tangential component * 2 + side.
template <int R, typename S, bool COH>
__device__ __forceinline__ void velocity_bc_point(const BcArgs<S> &a, int d, int sub, int i1, int i2, int zi) {
  typedef typename Storage<S>::C C;
  const Geom &g = a.g;
  int a1, a2;
  plane_axes(d, a1, a2);
  const int n1 = gdim(g, a1), n2 = gdim(g, a2), nd = gdim(g, d);
  if (i1 < 1 || i1 >= n1 - 1 || i2 < 1 || i2 >= n2 - 1) return;
  const int side = zi & 1;
  const int fb = a.face[2 * d + side];
  if (fb == 0) return;
  const int m = g.m;
  const int b = side == 0 ? m : nd - m - 1;
  const long base = plane_lin(g, d, i1, i2, 0);
  const long sd = gstride(g, d);
  const int comp = (sub == 0) ? d : ((zi >> 1) == 0 ? a1 : a2);
  const int F = F_U + comp;
  S *v = a.f1[F];
  if (fb == 2) {  // Robertsson
    const bool stag = (comp == d);
#pragma unroll
    for (int k = 0; k < R; ++k) {
      int idx;
      if (stag) idx = side == 0 ? b - 1 - k : b + k;
      else idx = side == 0 ? b - 1 - k : b + 1 + k;
      v[base + idx * sd] = Storage<S>::store(C(0), a.sc[F]);
    }
    return;
  }
  auto LD = [&](int f, long off) -> C { return Storage<S>::load(ldg<COH>(&a.f1[f][off]), a.inv[f]); };
  if (comp == d) {
    const long ob = base + b * sd;
    const C lam = (C)a.media[M_LAM][ob], mu = (C)a.media[M_MU][ob];
    const C r = lam / (lam + C(2) * mu);
    C s = 0;
#pragma unroll
    for (int t = 0; t < 2; ++t) {
      const int j = t == 0 ? a1 : a2;
      const long sj = gstride(g, j);
      s += (a.h[d] / a.h[j]) * (LD(F_U + j, ob) - LD(F_U + j, ob - sj));
    }
    if (side == 0)
      v[base + (b - 1) * sd] = Storage<S>::store(LD(F, ob) + r * s, a.sc[F]);
    else
      v[ob] = Storage<S>::store(LD(F, ob - sd) - r * s, a.sc[F]);
    return;
  }
  // tangential component v_j, j = comp
  const int j = comp;
  const long sj = gstride(g, j);
  const int Fd = F_U + d;
  const int mp = mu_pair(j, d);
  const long ob = base + b * sd, obm = ob - sd;
  const C mu_lo = (C)a.media[mp][obm], mu_hi = (C)a.media[mp][ob];
  const C hr = a.h[d] / a.h[j];
  const C Gm = hr * (LD(Fd, obm + sj) - LD(Fd, obm));   // G(b-1)
  const C G0 = hr * (LD(Fd, ob + sj) - LD(Fd, ob));     // G(b)
  if (side == 0) {
    const C val = LD(F, ob) + Gm - (mu_hi / mu_lo) * (LD(F, ob + sd) - LD(F, ob) + G0);
    v[obm] = Storage<S>::store(val, a.sc[F]);
  } else {
    const C val = LD(F, ob) - G0 + (mu_lo / mu_hi) * (LD(F, ob) - LD(F, obm) + Gm);
    v[ob + sd] = Storage<S>::store(val, a.sc[F]);
  }
}

// Levander ghost value of the component along d at in-plane point (i1, i2)
// of side `side` (the value velocity_bc_point writes for sub 0).
template <typename S, bool COH>
__device__ __forceinline__ typename Storage<S>::C levander_normal_ghost(const BcArgs<S> &a, int d, int side,
                                                                        int i1, int i2) {
  typedef typename Storage<S>::C C;
  const Geom &g = a.g;
  int a1, a2;
  plane_axes(d, a1, a2);
  const int nd = gdim(g, d);
  const int b = side == 0 ? g.m : nd - g.m - 1;
  const long sd = gstride(g, d);
  const long ob = plane_lin(g, d, i1, i2, 0) + b * sd;
  const int F = F_U + d;
  auto LD = [&](int f, long off) -> C { return Storage<S>::load(ldg<COH>(&a.f1[f][off]), a.inv[f]); };
  const C lam = (C)a.media[M_LAM][ob], mu = (C)a.media[M_MU][ob];
  const C r = lam / (lam + C(2) * mu);
  C s = 0;
#pragma unroll
  for (int t = 0; t < 2; ++t) {
    const int j = t == 0 ? a1 : a2;
    const long sj = gstride(g, j);
    s += (a.h[d] / a.h[j]) * (LD(F_U + j, ob) - LD(F_U + j, ob - sj));
  }
  return side == 0 ? LD(F, ob) + r * s : LD(F, ob - sd) - r * s;
}

// All velocity ghosts of face normal d at in-plane point (i1, i2): the
// component along d, then the two tangential components, which need the new
// along-d ghost at this point and at the next point along their own axis.
// That neighbour value is recomputed here from the same inputs (where the
// neighbour lies inside the along-d range) instead of read after another
// thread wrote it, so one launch per face normal gives the two-phase result.
template <int R, typename S, bool COH>
__device__ __forceinline__ void velocity_bc_merged_point(const BcArgs<S> &a, int d, int i1, int i2) {
  typedef typename Storage<S>::C C;
  const Geom &g = a.g;
  int a1, a2;
  plane_axes(d, a1, a2);
  const int n1 = gdim(g, a1), n2 = gdim(g, a2), nd = gdim(g, d);
  if (i1 < 1 || i1 >= n1 - 1 || i2 < 1 || i2 >= n2 - 1) return;
  const long sd = gstride(g, d);
  const int Fd = F_U + d;
  for (int side = 0; side < 2; ++side) {
    const int fb = a.face[2 * d + side];
    if (fb == 0) continue;
    if (fb == 2) {
      velocity_bc_point<R, S, COH>(a, d, 0, i1, i2, side);
      velocity_bc_point<R, S, COH>(a, d, 1, i1, i2, side);
      velocity_bc_point<R, S, COH>(a, d, 1, i1, i2, 2 + side);
      continue;
    }
    const int b = side == 0 ? g.m : nd - g.m - 1;
    const long base = plane_lin(g, d, i1, i2, 0);
    const long ob = base + b * sd, obm = ob - sd;
    const long gpos = side == 0 ? obm : ob;        // where the along-d ghost lives
    if constexpr (R == 2 && sizeof(S) <= 4) {
      if (a.gen) {
        // the generated ghost expressions; offsets are taken from plane b
        const float vg = gen_velocity_ghost(a, d, d, side, ghost_acc<S, COH>(a, ob));
        a.f1[Fd][gpos] = Storage<S>::store(vg, a.sc[Fd]);
        const float vg0 = Storage<S>::load(Storage<S>::store(vg, a.sc[Fd]), a.inv[Fd]);
        for (int t = 0; t < 2; ++t) {
          const int j = t == 0 ? a1 : a2;
          const long sj = gstride(g, j);
          // along-d ghost at the next point along j: recomputed where the
          // reference's face order has written it first, else the stored value
          const int n1j = t == 0 ? i1 + 1 : i1, n2j = t == 0 ? i2 : i2 + 1;
          const bool in = n1j >= 1 && n1j < n1 - 1 && n2j >= 1 && n2j < n2 - 1;
          const float vgn =
              in ? Storage<S>::load(Storage<S>::store(gen_velocity_ghost(a, d, d, side, ghost_acc<S, COH>(a, ob + sj)),
                                                      a.sc[Fd]), a.inv[Fd])
                 : (float)Storage<S>::load(ldg<COH>(&a.f1[Fd][gpos + sj]), a.inv[Fd]);
          GhostAcc<S, COH> A = ghost_acc<S, COH>(a, ob);
          A.fd = Fd;
          A.gd = d;
          A.gv = side == 0 ? -1 : 0;
          A.ja = j;
          A.v0 = vg0;
          A.vn = vgn;
          const int F = F_U + j;
          const float val = gen_velocity_ghost(a, j, d, side, A);
          a.f1[F][side == 0 ? obm : ob + sd] = Storage<S>::store(val, a.sc[F]);
        }
        continue;
      }
    }
    const C vg = levander_normal_ghost<S, COH>(a, d, side, i1, i2);
    a.f1[Fd][gpos] = Storage<S>::store(vg, a.sc[Fd]);
    auto LD = [&](int f, long off) -> C { return Storage<S>::load(ldg<COH>(&a.f1[f][off]), a.inv[f]); };
    for (int t = 0; t < 2; ++t) {
      const int j = t == 0 ? a1 : a2;
      const long sj = gstride(g, j);
      // along-d ghost at the next point along j: recomputed when the
      // two-phase order would have written it first, else the stored value
      const int n1j = t == 0 ? i1 + 1 : i1, n2j = t == 0 ? i2 : i2 + 1;
      const bool in = n1j >= 1 && n1j < n1 - 1 && n2j >= 1 && n2j < n2 - 1;
      const C vgn = in ? Storage<S>::load(Storage<S>::store(levander_normal_ghost<S, COH>(a, d, side, n1j, n2j),
                                                            a.sc[Fd]), a.inv[Fd])
                       : LD(Fd, gpos + sj);
      const C vg0 = Storage<S>::load(Storage<S>::store(vg, a.sc[Fd]), a.inv[Fd]);
      const int F = F_U + j;
      const int mp = mu_pair(j, d);
      const C mu_lo = (C)a.media[mp][obm], mu_hi = (C)a.media[mp][ob];
      const C hr = a.h[d] / a.h[j];
      if (side == 0) {
        const C Gm = hr * (vgn - vg0);                          // G(b-1), ghost plane
        const C G0 = hr * (LD(Fd, ob + sj) - LD(Fd, ob));        // G(b)
        const C val = LD(F, ob) + Gm - (mu_hi / mu_lo) * (LD(F, ob + sd) - LD(F, ob) + G0);
        a.f1[F][obm] = Storage<S>::store(val, a.sc[F]);
      } else {
        const C Gm = hr * (LD(Fd, obm + sj) - LD(Fd, obm));      // G(b-1)
        const C G0 = hr * (vgn - vg0);                          // G(b), ghost plane
        const C val = LD(F, ob) - G0 + (mu_lo / mu_hi) * (LD(F, ob) - LD(F, obm) + Gm);
        a.f1[F][ob + sd] = Storage<S>::store(val, a.sc[F]);
      }
    }
  }
}

// One launch per face normal; the first (d = 0) also applies the point
// source to the new stresses and advances the device step counter (step !=
// nullptr), which commutes with the velocity ghosts (disjoint arrays).  A
// captured step graph replays with unchanged arguments: the wavelet sample is
// picked on the device from the step counter.
template <int R, typename S>
__global__ void __launch_bounds__(256) velocity_bc_merged_kernel(const __grid_constant__ BcArgs<S> a, S *txx, S *tyy, S *tzz, long src_off,
                                                                 const float *w, int nt, long *step, float s0,
                                                                 float s1, float s2) {
  const int i2 = blockIdx.x * blockDim.x + threadIdx.x;
  const int i1 = blockIdx.y * blockDim.y + threadIdx.y;
  velocity_bc_merged_point<R, S, false>(a, a.d, i1, i2);
  if (step != nullptr && a.d == 0 && i1 == 0 && i2 == 0) {
    const long st = *step;
    if (src_off >= 0 && st < nt) {
      // w holds the x, y and z source signals, nt values each
      txx[src_off] = Storage<S>::store(Storage<S>::load(txx[src_off], 1.f / s0) - w[st] / 3, s0);
      tyy[src_off] = Storage<S>::store(Storage<S>::load(tyy[src_off], 1.f / s1) - w[nt + st] / 3, s1);
      tzz[src_off] = Storage<S>::store(Storage<S>::load(tzz[src_off], 1.f / s2) - w[2 * nt + st] / 3, s2);
    }
    *step = st + 1;
  }
}

// Velocity ghosts of face normal d with the generated ghost expressions
// (space order 4, BcArgs::gen) for one 32 x 8 block of in-plane points
// (i1, i2) = (by * 8 + ty, bx * 32 + tx): as velocity_bc_merged_point, but
// the block first computes the along-d component's ghost of its points and
// of the row and column beyond them into shared memory, once, and the
// tangential ghosts read the fresh values from there (the merged form
// evaluates each along-d ghost three times).  Robertsson faces as there.
// Every thread of the block calls it (it synchronises the block).
template <int R, typename S>
__device__ __forceinline__ void velocity_gen_block(const BcArgs<S> &a, int d, int i1, int i2) {
  if constexpr (R == 2 && sizeof(S) <= 4) {
    __shared__ float tile[9][33];
    const Geom &g = a.g;
    int a1, a2;
    plane_axes(d, a1, a2);
    const int n1 = gdim(g, a1), n2 = gdim(g, a2), nd = gdim(g, d);
    const int tx = threadIdx.x, ty = threadIdx.y;
    auto inrange = [&](int p1, int p2) { return p1 >= 1 && p1 < n1 - 1 && p2 >= 1 && p2 < n2 - 1; };
    const bool act = inrange(i1, i2);
    const long sd = gstride(g, d);
    const int Fd = F_U + d;
    for (int side = 0; side < 2; ++side) {
      const int fb = a.face[2 * d + side];   // the same for the whole block
      if (fb == 0) continue;
      if (fb == 2) {
        if (act) {
          velocity_bc_point<R, S, false>(a, d, 0, i1, i2, side);
          velocity_bc_point<R, S, false>(a, d, 1, i1, i2, side);
          velocity_bc_point<R, S, false>(a, d, 1, i1, i2, 2 + side);
        }
        continue;
      }
      const int b = side == 0 ? g.m : nd - g.m - 1;
      auto ob_of = [&](int p1, int p2) {
        return plane_lin(g, d, p1, p2, b);
      };
      auto fresh = [&](int p1, int p2) {
        const float v = gen_velocity_ghost(a, d, d, side, ghost_acc<S, false>(a, ob_of(p1, p2)));
        return (float)Storage<S>::load(Storage<S>::store(v, a.sc[Fd]), a.inv[Fd]);
      };
      const long ob = ob_of(i1, i2);
      const long gpos = side == 0 ? ob - sd : ob;
      float vg0 = 0.f;
      if (act) {
        const float vg = gen_velocity_ghost(a, d, d, side, ghost_acc<S, false>(a, ob));
        a.f1[Fd][gpos] = Storage<S>::store(vg, a.sc[Fd]);
        vg0 = (float)Storage<S>::load(Storage<S>::store(vg, a.sc[Fd]), a.inv[Fd]);
      }
      tile[ty][tx] = vg0;
      if (ty == 7) tile[8][tx] = inrange(i1 + 1, i2) ? fresh(i1 + 1, i2) : 0.f;
      if (tx == 31) tile[ty][32] = inrange(i1, i2 + 1) ? fresh(i1, i2 + 1) : 0.f;
      __syncthreads();
      if (act) {
        for (int t = 0; t < 2; ++t) {
          const int j = t == 0 ? a1 : a2;
          const long sj = gstride(g, j);
          // along-d ghost at the next point along j: the fresh value where the
          // reference's face order has written it first, else the stored one
          const bool in = t == 0 ? inrange(i1 + 1, i2) : inrange(i1, i2 + 1);
          const float vgn = in ? (t == 0 ? tile[ty + 1][tx] : tile[ty][tx + 1])
                               : (float)Storage<S>::load(a.f1[Fd][gpos + sj], a.inv[Fd]);
          GhostAcc<S, false> A = ghost_acc<S, false>(a, ob);
          A.fd = Fd;
          A.gd = d;
          A.gv = side == 0 ? -1 : 0;
          A.ja = j;
          A.v0 = vg0;
          A.vn = vgn;
          const int F = F_U + j;
          const float val = gen_velocity_ghost(a, j, d, side, A);
          a.f1[F][side == 0 ? ob - sd : ob + sd] = Storage<S>::store(val, a.sc[F]);
        }
      }
      __syncthreads();
    }
  }
}

// One launch per face normal with the generated ghost expressions; the
// first also applies the source and advances the step counter, as
// velocity_bc_merged_kernel.
template <int R, typename S>
__global__ void __launch_bounds__(256) velocity_bc_gen_kernel(const __grid_constant__ BcArgs<S> a, S *txx, S *tyy, S *tzz, long src_off,
                                                              const float *w, int nt, long *step, float s0, float s1,
                                                              float s2) {
  const int i2 = blockIdx.x * 32 + threadIdx.x, i1 = blockIdx.y * 8 + threadIdx.y;
  velocity_gen_block<R, S>(a, a.d, i1, i2);
  if (step != nullptr && a.d == 0 && i1 == 0 && i2 == 0) {
    const long st = *step;
    if (src_off >= 0 && st < nt) {
      // w holds the x, y and z source signals, nt values each
      txx[src_off] = Storage<S>::store(Storage<S>::load(txx[src_off], 1.f / s0) - w[st] / 3, s0);
      tyy[src_off] = Storage<S>::store(Storage<S>::load(tyy[src_off], 1.f / s1) - w[nt + st] / 3, s1);
      tzz[src_off] = Storage<S>::store(Storage<S>::load(tzz[src_off], 1.f / s2) - w[2 * nt + st] / 3, s2);
    }
    *step = st + 1;
  }
}

// ------------------------------------------------------------ receivers
// Seismogram sampling (tests/src/test_ref_iso_elastic.cpp:227-270 records
// U, V, W and the pressure (Txx + Tyy + Tzz) / 3 at each receiver every
// step): after a step's velocity ghosts and source, row (step counter - 1)
// of traces[cap][4][nrec] receives the values of level t1.  Steps beyond
// the buffer's capacity are not recorded.
template <typename S>
struct RecArgs {
  const S *f[6];       // U V W Txx Tyy Tzz at level t1
  float inv[6];        // 1 / storage scale
  const long *rec;     // element offsets of the receivers
  int nrec, cap;
  float *traces;
  const long *step;    // device step counter, already advanced
};

// COH: read through L2 only (values written by other CTAs of the same launch)
template <bool COH, typename S>
__device__ __forceinline__ void sample_receiver_at(const RecArgs<S> &r, long row, int i) {
  typedef typename Storage<S>::C C;
  const long o = r.rec[i];
  float *t = r.traces + row * 4 * (long)r.nrec;
  auto L = [&](int k) -> C { return (C)Storage<S>::load(ldg<COH>(&r.f[k][o]), r.inv[k]); };
  t[i] = (float)L(0);
  t[r.nrec + i] = (float)L(1);
  t[2 * r.nrec + i] = (float)L(2);
  const C p = (L(3) + L(4) + L(5)) / 3;
  t[3 * r.nrec + i] = (float)p;
}

template <typename S>
__device__ __forceinline__ void sample_receiver(const RecArgs<S> &r, long row, int i) {
  sample_receiver_at<false>(r, row, i);
}

template <typename S>
__device__ __forceinline__ void sample_receiver_coherent(const RecArgs<S> &r, long row, int i) {
  sample_receiver_at<true>(r, row, i);
}

template <typename S>
__global__ void receiver_sample_kernel(RecArgs<S> r) {
  const long row = *r.step - 1;
  if (row < 0 || row >= r.cap) return;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < r.nrec; i += gridDim.x * blockDim.x)
    sample_receiver(r, row, i);
}

// ------------------------------------------------------- grouped launches
// One launch per face normal covers the ghost work of every member of a
// group: each member owns a contiguous range of the launch's 32 x 8 blocks
// (its own face grid, flattened), found by binary search.
template <typename S>
struct GroupBc {
  BcArgs<S> a;
  int begin[3];        // first block of this member in the launch for face normal d
  int bx[3], by[3];    // the member's face grid for face normal d
  // point source and step counter (velocity ghosts, face normal 0)
  S *txx, *tyy, *tzz;
  long src_off;        // -1: no source
  const float *w;
  int nt;
  long *step;
  float s0, s1, s2;
  RecArgs<S> rec;      // receivers of the member (nrec = 0: none)
  int rbegin, rbx, rby; // generated-recompute launch: first block, 32 x 4 block grid of a face
};

template <typename S>
__device__ __forceinline__ int group_bc_member(const GroupBc<S> *tab, int n, int d) {
  __shared__ int s_member;
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (tab[mid].begin[d] <= (int)blockIdx.x) lo = mid;
      else hi = mid - 1;
    }
    s_member = lo;
  }
  __syncthreads();
  return s_member;
}

// blockIdx.x -> member; within the member z = field(0..5)*2 + side
template <int R, typename S>
__global__ void __launch_bounds__(256) stress_bc_group_kernel(const GroupBc<S> *__restrict__ tab, int n, int d) {
  const GroupBc<S> &e = tab[group_bc_member(tab, n, d)];
  const int local = (int)blockIdx.x - e.begin[d];
  const int per = e.bx[d] * e.by[d];
  const int z = local / per, r = local - z * per;
  const int i2 = (r % e.bx[d]) * 32 + threadIdx.x;
  const int i1 = (r / e.bx[d]) * 8 + threadIdx.y;
  stress_bc_point<R, S, false>(e.a, d, i1, i2, z >> 1, z & 1);
}

template <int R, typename S>
__global__ void __launch_bounds__(256) velocity_bc_group_kernel(const GroupBc<S> *__restrict__ tab, int n, int d) {
  const GroupBc<S> &e = tab[group_bc_member(tab, n, d)];
  const int local = (int)blockIdx.x - e.begin[d];
  const int i2 = (local % e.bx[d]) * 32 + threadIdx.x;
  const int i1 = (local / e.bx[d]) * 8 + threadIdx.y;
  if (e.a.gen) velocity_gen_block<R, S>(e.a, d, i1, i2);   // uniform in the block
  else velocity_bc_merged_point<R, S, false>(e.a, d, i1, i2);
  if (d == 0 && local == 0 && threadIdx.x == 0 && threadIdx.y == 0 && e.step != nullptr) {
    const long st = *e.step;
    if (e.src_off >= 0 && st < e.nt) {
      const long o = e.src_off;
      e.txx[o] = Storage<S>::store(Storage<S>::load(e.txx[o], 1.f / e.s0) - e.w[st] / 3, e.s0);
      e.tyy[o] = Storage<S>::store(Storage<S>::load(e.tyy[o], 1.f / e.s1) - e.w[e.nt + st] / 3, e.s1);
      e.tzz[o] = Storage<S>::store(Storage<S>::load(e.tzz[o], 1.f / e.s2) - e.w[2 * e.nt + st] / 3, e.s2);
    }
    *e.step = st + 1;
  }
}

// Generated normal-stress recompute values of every member that has them
// (BcArgs::rc set), as stress_recompute_kernel: grid-stride over virtual
// 32 x 4 blocks (member ranges from rbegin, each member's grid rbx x rby x 12).
template <int R, typename S>
__global__ void __launch_bounds__(128, 12) stress_recompute_group_kernel(const GroupBc<S> *__restrict__ tab, int n,
                                                                     int total) {
  if constexpr (R == 2 && sizeof(S) <= 4) {
    for (int vb = blockIdx.x; vb < total; vb += gridDim.x) {
      int lo = 0, hi = n - 1;
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (tab[mid].rbegin <= vb) lo = mid;
        else hi = mid - 1;
      }
      const GroupBc<S> &e = tab[lo];
      const BcArgs<S> &a = e.a;
      if (!a.rc) continue;
      const int local = vb - e.rbegin;
      const int per = e.rbx * e.rby;
      if (local >= per * 12) continue;
      const int z = local / per, r = local - z * per;
      const Geom &g = a.g;
      const int q = z & 1, side = (z >> 1) & 1, d = z >> 2;
      int a1, a2;
      plane_axes(d, a1, a2);
      const int n1 = gdim(g, a1), n2 = gdim(g, a2), nd = gdim(g, d);
      const int i2 = (r % e.rbx) * 32 + threadIdx.x;
      const int i1 = (r / e.rbx) * 4 + threadIdx.y;
      const int m = g.m;
      if (i1 < m + 1 || i1 >= n1 - m - 1 || i2 < m + 1 || i2 >= n2 - m - 1) continue;
      if (a.face[2 * d + side] != 1) continue;
      const int fi = q < d ? q : q + 1;
      const int b = side == 0 ? m : nd - m - 1;
      const auto A = ghost_acc<S, false>(a, plane_lin(g, d, i1, i2, b));
      const float v =
          gen_stress_recompute(a, fi, d, side, A);
      const_cast<float *>(a.rc)[(long)z * a.rcs + (long)i1 * n2 + i2] = v;
    }
  }
}

// receivers of every member: block = member
template <typename S>
__global__ void receiver_sample_group_kernel(const GroupBc<S> *__restrict__ tab) {
  const RecArgs<S> &r = tab[blockIdx.x].rec;
  if (r.nrec <= 0) return;
  const long row = *r.step - 1;
  if (row < 0 || row >= r.cap) return;
  for (int i = threadIdx.x; i < r.nrec; i += blockDim.x) sample_receiver(r, row, i);
}

}  // namespace ofd
