// Tiled stress / velocity sweeps for sm_103a: 2.5D blocking with TMA.
//
// A CTA owns a TZ x TY tile of the two fast axes (z contiguous, y) and walks a
// chunk of planes along the slow axis x.  Every plane of the arrays the update
// reads with neighbours ("halo" arrays: U V W for the stress sweep, the six
// stresses for the velocity sweep) arrives in shared memory as one TMA box of
// (TZ + 2 ZH) x (TY + 2R) elements; a ring of NSH such planes holds the x
// window [x-R, x+R] plus the planes in flight.  Arrays read only at the point
// (the field being updated at t0, the media) arrive as TZ x TY boxes in a
// second ring of NSC planes.  Each ring slot has an mbarrier; one thread
// issues cp.async.bulk.tensor loads with complete_tx accounting, everyone
// else waits on the slot's phase (bounded: a wait that runs out sets the
// error word and the CTA drains its loads and returns).  Results go straight
// to HBM with coalesced 128-byte row stores.
//
// The arithmetic is the generated expression (GenSweep) read through an
// accessor that maps A(f, dx, dy, dz) onto the rings, so the tiled kernels
// compute bit for bit what the plain kernels compute.
#pragma once
#include <cuda.h>
#include "ofd_common.cuh"
#include "generated/sweeps_gen.cuh"

namespace ofd {

constexpr int TZ = 64;          // tile width along z (two 32-lane passes)
constexpr int TY = 8;           // tile height along y (one warp per row)
constexpr int TILED_THREADS = TZ / 2 * TY;   // 256: warp w -> row w, lane l -> z = l, l+32

template <typename S> struct ZHalo { static constexpr int v = (int)(16 / sizeof(S)) >= 4 ? (int)(16 / sizeof(S)) : 4; };

// TMA descriptors of one handle: per field and level a halo box and a point
// box, per media array a point box.
struct TmaMaps {
  CUtensorMap halo[9][2];
  CUtensorMap point[9][2];
  CUtensorMap media[8];
  int ok;
};

// Host-side context of a handle for the tiled launches.
struct TiledCtx {
  const TmaMaps *maps;   // nullptr: descriptors unavailable, use plain kernels
  int *err;              // device error word
  int z0;                // element offset of z = 0 in a padded row
};

// Box extents the runtime encodes into the descriptors.
inline void tiled_boxes(int R, int esize, int *hw, int *hh, int *pw, int *ph) {
  const int zh = (16 / esize) >= 4 ? 16 / esize : 4;
  *hw = TZ + 2 * zh;
  *hh = TY + 2 * R;
  *pw = TZ;
  *ph = TY;
}

struct TiledParams {
  CUtensorMap hmap[6];     // halo arrays in order of hfield[]
  CUtensorMap pmap[6];     // point field arrays in order of pfield[]
  CUtensorMap mmap[5];     // media arrays in order of mfield[]
  int *err;                // error word (bounded waits)
  int zcoord0;             // TMA x coordinate of z = m (z0 + m)
  int chunk;               // planes per CTA along x
  int ntz, nty;            // tiles along z, y
};

__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait; false when the limit ran out.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity) {
  for (long it = 0; it < (1L << 24); ++it)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, uint64_t *bar, int c0, int c1, int c2) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5}], [%2];"
      ::"r"(smem_u32(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(c0), "r"(c1), "r"(c2)
      : "memory");
}

__host__ __device__ constexpr int round128(int b) { return (b + 127) / 128 * 128; }

// Compile-time description of one sweep.
template <int R, typename S, int HET, bool STRESS>
struct TiledCfg {
  static constexpr int ZH = ZHalo<S>::v;                  // z halo, rounded to 16 B
  static constexpr int HW = TZ + 2 * ZH;                   // halo box width
  static constexpr int HH = TY + 2 * R;                    // halo box height
  static constexpr int NHF = STRESS ? 3 : 6;               // halo arrays
  static constexpr int NPF = STRESS ? 6 : 3;               // point field arrays
  static constexpr int NMF = HET ? (STRESS ? 5 : 3) : 0;   // point media arrays
  static constexpr int PF = 1;                             // planes prefetched ahead
  static constexpr int NSH = 2 * R + 1 + PF;               // halo ring depth
  static constexpr int NSC = 1 + PF;                       // point ring depth
  static constexpr int HBOX = HW * HH * (int)sizeof(S);
  static constexpr int HSLOT = round128(HBOX);
  static constexpr int PBOX = TZ * TY * (int)sizeof(S);
  static constexpr int MBOX = TZ * TY * 4;
  static constexpr int HRING = NSH * NHF * HSLOT;
  static constexpr int PRING = NSC * NPF * round128(PBOX);
  static constexpr int MRING = NSC * (NMF > 0 ? NMF : 1) * round128(MBOX);
  static constexpr int BARS = (NSH + NSC) * 8;
  static constexpr int SMEM = HRING + PRING + MRING + round128(BARS) + 128;  // +128: base alignment
  // field id -> slot in the halo / point lists
  __host__ __device__ static constexpr int hidx(int f) { return STRESS ? (f - F_U) : (f - F_TXX); }
  __host__ __device__ static constexpr int pidx(int f) { return STRESS ? (f - F_TXX) : (f - F_U); }
  __host__ __device__ static constexpr bool is_halo(int f) { return STRESS ? (f < F_TXX) : (f >= F_TXX); }
  __host__ __device__ static constexpr int midx(int m) {
    return STRESS ? (m - M_LAM) : (m - M_B1);
  }
};

template <int R, typename S, int HET, bool STRESS>
struct TiledAcc {
  typedef TiledCfg<R, S, HET, STRESS> G;
  typedef typename Storage<S>::C C;
  const S *hring;     // halo ring base
  const S *pring;
  const float *mring;
  const float *inv;
  int x, hq0;         // current plane, halo-ring plane origin (plane of q = 0)
  int pq0;
  int yl, zl;         // thread row / column in the tile
  __device__ __forceinline__ C operator()(int f, int dx, int dy, int dz) const {
    if (G::is_halo(f)) {
      const int q = x + dx - hq0;
      const int slot = q % G::NSH;
      const S *b = (const S *)((const char *)hring + (slot * G::NHF + G::hidx(f)) * G::HSLOT);
      return (C)Storage<S>::load(b[(yl + R + dy) * G::HW + (zl + G::ZH + dz)], inv[f]);
    }
    const int q = x - pq0;
    const int slot = q % G::NSC;
    const S *b = (const S *)((const char *)pring + (slot * G::NPF + G::pidx(f)) * round128(G::PBOX));
    return (C)Storage<S>::load(b[yl * TZ + zl], inv[f]);
  }
  __device__ __forceinline__ C m(int i) const {
    const int q = x - pq0;
    const int slot = q % G::NSC;
    const float *b = (const float *)((const char *)mring + (slot * (G::NMF > 0 ? G::NMF : 1) + G::midx(i)) * round128(G::MBOX));
    return (C)b[yl * TZ + zl];
  }
};

template <int R, typename S, int HET, bool STRESS>
__global__ void __launch_bounds__(TILED_THREADS)
sweep_tiled(const __grid_constant__ SweepArgs<S> a, const __grid_constant__ TiledParams p) {
  typedef TiledCfg<R, S, HET, STRESS> G;
  typedef typename Storage<S>::C C;
  extern __shared__ unsigned char smem_raw[];
  unsigned char *smem = (unsigned char *)(((uintptr_t)smem_raw + 127) & ~(uintptr_t)127);
  S *hring = (S *)smem;
  S *pring = (S *)(smem + G::HRING);
  float *mring = (float *)(smem + G::HRING + G::PRING);
  uint64_t *hbar = (uint64_t *)(smem + G::HRING + G::PRING + G::MRING);
  uint64_t *pbar = hbar + G::NSH;
  __shared__ int abort_flag;

  const Geom &g = a.g;
  const int tz = blockIdx.x % p.ntz, ty = blockIdx.x / p.ntz;
  const int z0 = g.m + tz * TZ, y0 = g.m + ty * TY;
  const int xb = g.m + blockIdx.y * p.chunk;
  const int xe = min(xb + p.chunk, g.n1 - g.m);
  if (xb >= xe) return;
  const int hq0 = xb - R;          // plane of halo q = 0
  const int hlast = xe - 1 + R;    // last halo plane needed
  const int tid = threadIdx.x;
  const int zc = p.zcoord0 + (z0 - g.m);

  auto issue_halo = [&](int plane) {
    const int q = plane - hq0;
    const int slot = q % G::NSH;
    uint64_t *bar = &hbar[slot];
    mbar_expect_tx(bar, G::NHF * G::HBOX);
#pragma unroll
    for (int i = 0; i < G::NHF; ++i)
      tma_load_3d((char *)hring + (slot * G::NHF + i) * G::HSLOT, &p.hmap[i], bar, zc - G::ZH, y0 - R, plane);
  };
  auto issue_point = [&](int plane) {
    const int q = plane - xb;
    const int slot = q % G::NSC;
    uint64_t *bar = &pbar[slot];
    mbar_expect_tx(bar, G::NPF * G::PBOX + G::NMF * G::MBOX);
#pragma unroll
    for (int i = 0; i < G::NPF; ++i)
      tma_load_3d((char *)pring + (slot * G::NPF + i) * round128(G::PBOX), &p.pmap[i], bar, zc, y0, plane);
#pragma unroll
    for (int i = 0; i < G::NMF; ++i)
      tma_load_3d((char *)mring + (slot * G::NMF + i) * round128(G::MBOX), &p.mmap[i], bar, zc, y0, plane);
  };

  int hissued = hq0 - 1, pissued = xb - 1;   // last plane issued (thread 0)
  if (tid == 0) {
    abort_flag = 0;
    for (int i = 0; i < G::NSH; ++i) mbar_init(&hbar[i], 1);
    for (int i = 0; i < G::NSC; ++i) mbar_init(&pbar[i], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    for (int pl = hq0; pl <= hlast && pl < hq0 + G::NSH; ++pl) { issue_halo(pl); hissued = pl; }
    for (int pl = xb; pl < xe && pl < xb + G::NSC; ++pl) { issue_point(pl); pissued = pl; }
  }
  __syncthreads();

  const int yl = tid >> 5, lane = tid & 31;
  const int y = y0 + yl;
  int hwaited = hq0 - 1;   // last halo plane waited for
  int pwaited = xb - 1;    // last point plane waited for
  bool ok = true;
  for (int x = xb; x < xe && ok; ++x) {
    // halo planes up to x + R, point plane x
    for (int pl = hwaited + 1; pl <= x + R && ok; ++pl) {
      const int q = pl - hq0;
      if (!mbar_wait(&hbar[q % G::NSH], (unsigned)((q / G::NSH) & 1))) ok = false;
      else hwaited = pl;
    }
    if (ok) {
      const int q = x - xb;
      if (!mbar_wait(&pbar[q % G::NSC], (unsigned)((q / G::NSC) & 1))) ok = false;
      else pwaited = x;
    }
    if (!ok) {
      atomicExch(p.err, 1);
      abort_flag = 1;
    }
    __syncthreads();
    if (abort_flag) break;
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      const int zl = lane + 32 * half;
      const int z = z0 + zl;
      TiledAcc<R, S, HET, STRESS> A{hring, pring, mring, a.inv, x, hq0, xb, yl, zl};
      const long o = (long)x * g.plane + (long)y * g.P + z;
      const bool inside = (z < g.n3 - g.m) && (y < g.n2 - g.m);
      if (STRESS) {
        C out[6];
        GenSweep<R, HET>::template stress<C>(A, a.K, out);
        if (inside) {
#pragma unroll
          for (int i = 0; i < 6; ++i) a.out[F_TXX + i][o] = Storage<S>::store(out[i], a.sc[F_TXX + i]);
        }
      } else {
        C out[3];
        GenSweep<R, HET>::template velocity<C>(A, a.K, out);
        if (inside) {
#pragma unroll
          for (int i = 0; i < 3; ++i) a.out[F_U + i][o] = Storage<S>::store(out[i], a.sc[F_U + i]);
        }
      }
    }
    __syncthreads();   // ring slots of plane x - R (halo) and x (point) are free
    if (tid == 0) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      const int nh = x - R + G::NSH;
      if (nh <= hlast) { issue_halo(nh); hissued = nh; }
      const int np = x + G::NSC;
      if (np < xe) { issue_point(np); pissued = np; }
    }
  }
  if (abort_flag && tid == 0) {
    // drain the loads this CTA issued and has not seen complete (bounded)
    for (int pl = hwaited + 1; pl <= hissued; ++pl) {
      const int q = pl - hq0;
      mbar_wait(&hbar[q % G::NSH], (unsigned)((q / G::NSH) & 1));
    }
    for (int pl = pwaited + 1; pl <= pissued; ++pl) {
      const int q = pl - xb;
      mbar_wait(&pbar[q % G::NSC], (unsigned)((q / G::NSC) & 1));
    }
  }
}

// ---------------------------------------------------------------- host side

template <int R, typename S, int HET, bool STRESS>
static bool tiled_fits() {
  return TiledCfg<R, S, HET, STRESS>::SMEM <= 227 * 1024 && TiledCfg<R, S, HET, STRESS>::HH <= 256;
}

template <int R, typename S>
bool tiled_supported(const Geom &g) {
  // the tiled path needs at least one full tile of interior along y and z
  if (g.n3 - 2 * g.m < TZ / 2 || g.n2 - 2 * g.m < TY) return false;
  return tiled_fits<R, S, 1, true>() && tiled_fits<R, S, 1, false>() && tiled_fits<R, S, 0, true>() &&
         tiled_fits<R, S, 0, false>();
}

template <int R, typename S, int HET, bool STRESS>
void launch_tiled(const SweepArgs<S> &a, const TiledCtx &ctx, int t0, cudaStream_t st) {
  typedef TiledCfg<R, S, HET, STRESS> G;
  const TmaMaps *mp = ctx.maps;
  const Geom &g = a.g;
  TiledParams p;
  const int t1 = 1 - t0;
  if (STRESS) {
    for (int i = 0; i < 3; ++i) p.hmap[i] = mp->halo[F_U + i][t0];
    for (int i = 0; i < 6; ++i) p.pmap[i] = mp->point[F_TXX + i][t0];
    for (int i = 0; i < 5; ++i) p.mmap[i] = mp->media[M_LAM + i];
  } else {
    for (int i = 0; i < 6; ++i) p.hmap[i] = mp->halo[F_TXX + i][t1];
    for (int i = 0; i < 3; ++i) p.pmap[i] = mp->point[F_U + i][t0];
    for (int i = 0; i < 3; ++i) p.mmap[i] = mp->media[M_B1 + i];
  }
  p.err = ctx.err;
  p.zcoord0 = ctx.z0 + g.m;
  const int nx = g.n1 - 2 * g.m, ny = g.n2 - 2 * g.m, nz = g.n3 - 2 * g.m;
  p.ntz = (nz + TZ - 1) / TZ;
  p.nty = (ny + TY - 1) / TY;
  const long tiles = (long)p.ntz * p.nty;
  // enough CTAs for ~8 waves of 152 SMs at the resident count, chunks >= 16 planes
  const int per_sm = (227 * 1024) / (G::SMEM + 1024) > 0 ? (227 * 1024) / (G::SMEM + 1024) : 1;
  long want = 152L * per_sm * 8;
  int chunks = (int)((want + tiles - 1) / tiles);
  if (chunks > nx / 16) chunks = nx / 16;
  if (chunks < 1) chunks = 1;
  p.chunk = (nx + chunks - 1) / chunks;
  chunks = (nx + p.chunk - 1) / p.chunk;
  auto kern = sweep_tiled<R, S, HET, STRESS>;
  cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, G::SMEM);
  kern<<<dim3((unsigned)tiles, (unsigned)chunks), TILED_THREADS, G::SMEM, st>>>(a, p);
}

template <int R, typename S, int HET>
void launch_stress_tiled(const SweepArgs<S> &a, const TiledCtx &c, int t0, cudaStream_t st) {
  launch_tiled<R, S, HET, true>(a, c, t0, st);
}
template <int R, typename S, int HET>
void launch_velocity_tiled(const SweepArgs<S> &a, const TiledCtx &c, int t0, cudaStream_t st) {
  launch_tiled<R, S, HET, false>(a, c, t0, st);
}

}  // namespace ofd
