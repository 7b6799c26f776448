// Tiled stress / velocity sweeps for sm_103a: 2.5D blocking with TMA.
//
// A CTA owns a TZ x TY tile of the two fast axes (z contiguous, y) and walks a
// chunk of planes along the slow axis x.  Every plane of the arrays the update
// reads with neighbours ("halo" arrays: U V W for the stress sweep, the six
// stresses for the velocity sweep) arrives in shared memory as one TMA box of
// (TZ + 2 ZH) x (TY + 2R) elements; a ring of NSH such planes holds the x
// window [x-R, x+R] plus the planes in flight.  Arrays read only at the point
// (the field being updated at t0, the media) arrive as TZ x TY boxes in a
// second ring of NSC planes.  The CTA is warp-specialised: one producer warp
// (lane 0) issues the cp.async.bulk.tensor loads, each slot with a "full"
// mbarrier (complete_tx accounting) and an "empty" mbarrier that the eight
// consumer warps (one per tile row) arrive on when they are done with the
// plane; the producer refills a slot once it is empty.  Consumers therefore
// wait only for their data, never for each other (no CTA-wide barrier per
// plane).  Every wait is bounded: one that runs out sets the error word and
// the CTA's abort flag, the other warps leave their loops, and the producer
// drains the loads in flight before the CTA exits.  Results go straight to
// HBM with coalesced 128-byte row stores.
//
// The arithmetic is the generated expression (GenSweep) read through an
// accessor that maps A(f, dx, dy, dz) onto the rings, so the tiled kernels
// compute bit for bit what the plain kernels compute.
#pragma once
#include <cuda.h>
#include "ofd_common.cuh"
#include "generated/sweeps_gen.cuh"
#include "ofd_f32x2.cuh"

namespace ofd {

constexpr int TZ = 64;          // tile width along z (two 32-lane passes)
// tile height along y (one warp per row).  Eight rows let two CTAs share an SM
// (measured faster than one CTA of sixteen rows, despite the extra halo rows)
__host__ __device__ constexpr int tile_rows(int) { return 8; }
// consumer warps per tile row: one warp covering the row's 64 z points in two
// 32-lane halves, or (space order >= 6, whose rings leave room for one CTA per
// SM) two warps of one point per lane, doubling the warps that hide latency
__host__ __device__ constexpr int row_warps(int R) { return R >= 3 ? 2 : 1; }

template <typename S> struct ZHalo { static constexpr int v = (int)(16 / sizeof(S)) >= 4 ? (int)(16 / sizeof(S)) : 4; };

// TMA descriptors of one handle: per field and level a halo box and a point
// box, per media array a point box.
struct TmaMaps {
  CUtensorMap halo[9][2];
  CUtensorMap point[9][2];
  CUtensorMap media[NM];
  CUtensorMap beta;      // (TZ + 4) x (TY + 1) boxes of beta: the point, y + 1 and z + 1
  int ok;
};

// Host-side context of a handle for the tiled launches.
struct TiledCtx {
  const TmaMaps *maps;   // nullptr: descriptors unavailable, use plain kernels
  int *err;              // device error word
  int z0;                // element offset of z = 0 in a padded row
  int waves;             // CTA-count multiplier (autotuner knob), 1 = default
  int kd[2];             // [stress]: the literal table follows KMap (register-held literals)
  unsigned long long wait_ns;   // limit of each pipeline wait
};

// Box extents the runtime encodes into the descriptors.
inline void beta_box(int R, int *bw, int *bh) {
  *bw = TZ + 4;
  *bh = tile_rows(R) + 1;
}

inline void tiled_boxes(int R, int esize, int *hw, int *hh, int *pw, int *ph) {
  const int zh = (16 / esize) >= 4 ? 16 / esize : 4;
  *hw = TZ + 2 * zh;
  *hh = tile_rows(R) + 2 * R;
  *pw = TZ;
  *ph = tile_rows(R);
}

struct TiledParams {
  CUtensorMap hmap[6];     // halo boxes: x-window arrays, then plane-halo arrays
  CUtensorMap pmap[6];     // point boxes of field arrays
  CUtensorMap mmap[5];     // point boxes of media arrays
  CUtensorMap bmap;        // beta boxes (heterogeneous velocity sweep)
  CUtensorMap xpmap[3];    // point boxes of the x-window arrays (split staging)
  int *err;                // error word (bounded waits)
  unsigned long long wait_ns;   // limit of each pipeline wait (ns of %globaltimer)
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

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}

// Bounded wait; false when 10 s of wall time ran out (a time bound, not an
// iteration count, so heavy concurrent load never trips it spuriously).  Used
// by the drain after an abort, which waits for copies already in flight.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = global_ns();
  for (;;) {
    for (int i = 0; i < 64; ++i)
      if (mbar_try_wait(bar, parity)) return true;
    if (global_ns() - t0 > 10000000000ULL) return false;
  }
}

// Bounded wait of the pipeline (limit_ns of wall time, the handle's wait
// limit) that also returns false once another warp of the CTA has aborted
// (*abort != 0).
__device__ __forceinline__ bool mbar_wait_or_abort(uint64_t *bar, unsigned parity, volatile int *abort,
                                                   unsigned long long limit_ns) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = global_ns();
  for (;;) {
    for (int i = 0; i < 64; ++i)
      if (mbar_try_wait(bar, parity)) return true;
    if (*abort) return false;
    if (global_ns() - t0 > limit_ns) return false;
  }
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, uint64_t *bar, int c0, int c1, int c2) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5}], [%2];"
      ::"r"(smem_u32(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(c0), "r"(c1), "r"(c2)
      : "memory");
}

__host__ __device__ constexpr int round128(int b) { return (b + 127) / 128 * 128; }

// Paired evaluation (ofd_f32x2.cuh): heterogeneous media and FP32 arithmetic
// (FP32, FP16 or BF16 storage).  Each consumer lane then owns two adjacent z
// points and one warp covers a 64-point tile row.  The literal table is then
// passed as pairs {K, K} (KRegs2 or KPairPtr below).
template <typename S, int HET> struct PairMode {
  static constexpr bool v = HET != 0 && sizeof(S) <= 4;
};

// Compile-time description of one sweep.  Roles of the arrays read:
//   X  ("x-window"): read at x offsets and with y/z neighbours (stress: U V W;
//      velocity: Txx Txy Txz)
//   H  ("plane halo"): y/z neighbours at the current plane only (velocity:
//      Tyy Tyz Tzz) -> halo boxes in the plane ring
//   P  (point): the value at the point (stress: the six stresses at t0;
//      velocity: U V W at t0) and the media arrays -> point boxes in the
//      plane ring (NSC planes)
// An X array is staged in one of two ways:
//   * whole (SPLIT false, space order <= 4): every plane of the x window as a
//     halo box in the x-window ring (NSH planes);
//   * split (SPLIT true, space order >= 6): the update reads an X array
//     either at an x offset (dy = dz = 0) or with a y/z neighbour at the
//     current plane (dx = 0), never both (the generated expressions mix no
//     offsets), so the x-window ring holds point boxes only and the current
//     plane's halo box of each X array read with y/z neighbours goes to the
//     plane ring.  The halo box re-reads the point values from L2 (they were
//     fetched R planes earlier); the rings shrink enough to keep two or three
//     planes in flight (PF), which these orders need to cover DRAM latency.
template <int R, typename S, int HET, bool STRESS>
struct TiledCfg {
  static constexpr bool PAIR = PairMode<S, HET>::v;
  static constexpr bool SPLIT = R >= 3;
  static constexpr int TY = tile_rows(R);
  static constexpr int ZW = PAIR ? 1 : row_warps(R);       // consumer warps per tile row
  static constexpr int NCW = TY * ZW;                      // consumer warps
  static constexpr int THREADS = 32 * (NCW + 1);           // + one producer warp
  static constexpr int ZH = ZHalo<S>::v;                  // z halo, rounded to 16 B
  static constexpr int HW = TZ + 2 * ZH;                   // halo box width
  static constexpr int HH = TY + 2 * R;                    // halo box height
  static constexpr int NXF = 3;                            // x-window arrays
  // current-plane halo boxes of X arrays (split staging): stress U V W,
  // velocity Txy Txz (Txx is read at x offsets only)
  static constexpr int NXH = SPLIT ? (STRESS ? 3 : 2) : 0;
  static constexpr int NH0 = STRESS ? 0 : 3;               // plane-halo arrays
  static constexpr int NPF = STRESS ? 6 : 3;               // point field arrays
  // point media arrays: lambda mu mu12 mu13 mu23 (stress).  The velocity
  // sweep reads beta instead of beta1..3, as one box per x-window plane
  // covering the point, y + 1 and z + 1 (z extent rounded to 16 bytes), and
  // averages on the fly exactly as the media preprocessing does.
  static constexpr int NMF = (HET && STRESS) ? 5 : 0;
  static constexpr int NBX = (HET && !STRESS) ? 1 : 0;    // beta box per x-window plane
  static constexpr int BW = TZ + 4, BH = TY + 1;          // beta box extent (floats)
  // planes prefetched ahead: split FP32 staging keeps one CTA per SM with
  // three planes in flight; 16-bit storage halves the boxes, so two planes in
  // flight still leave room for two CTAs per SM
  static constexpr int PF = SPLIT ? (sizeof(S) <= 2 ? 2 : 3) : 1;
  static constexpr int NSH = 2 * R + 1 + PF;               // x-window ring depth
  static constexpr int NSC = 1 + PF;                       // plane ring depth
  static constexpr int HBOX = HW * HH * (int)sizeof(S);
  static constexpr int HSLOT = round128(HBOX);
  static constexpr int PBOX = TZ * TY * (int)sizeof(S);
  static constexpr int PSLOT = round128(PBOX);
  static constexpr int MBOX = TZ * TY * 4;
  static constexpr int MSLOT = round128(MBOX);
  static constexpr int XBOX = SPLIT ? PBOX : HBOX;         // box of an X array in the x-window ring
  static constexpr int XSLOT = SPLIT ? PSLOT : HSLOT;
  // one x-window ring stage holds NXF X boxes (+ the beta box); one plane
  // ring stage holds NXH + NH0 halo boxes, NPF point boxes and NMF media boxes
  static constexpr int BBOX = BW * BH * 4;
  static constexpr int BSLOT = round128(BBOX);
  static constexpr int XSTAGE = NXF * XSLOT + NBX * BSLOT;
  static constexpr int CSTAGE = (NXH + NH0) * HSLOT + NPF * PSLOT + NMF * MSLOT;
  static constexpr int XRING = NSH * XSTAGE;
  static constexpr int CRING = NSC * CSTAGE;
  static constexpr int BARS = 2 * (NSH + NSC) * 8;        // full and empty barrier per slot
  static constexpr int SMEM = XRING + CRING + round128(BARS) + 128;  // +128: base alignment
  static constexpr unsigned XBYTES = NXF * XBOX + NBX * BBOX;
  static constexpr unsigned CBYTES = (NXH + NH0) * HBOX + NPF * PBOX + NMF * MBOX;
  // role and index of a field id
  __host__ __device__ static constexpr int role(int f) {   // 0 X, 1 H, 2 P
    return STRESS ? (f < F_TXX ? 0 : 2)
                  : (f < F_TXX ? 2 : ((f == F_TXX || f == F_TXY || f == F_TXZ) ? 0 : 1));
  }
  __host__ __device__ static constexpr int xidx(int f) {
    return STRESS ? (f - F_U) : (f == F_TXX ? 0 : (f == F_TXY ? 1 : 2));
  }
  // index among the current-plane halo boxes of X arrays (split staging)
  __host__ __device__ static constexpr int xhidx(int f) { return STRESS ? (f - F_U) : (f == F_TXY ? 0 : 1); }
  __host__ __device__ static constexpr int h0idx(int f) { return f == F_TYY ? 0 : (f == F_TYZ ? 1 : 2); }
  __host__ __device__ static constexpr int pidx(int f) { return STRESS ? (f - F_TXX) : (f - F_U); }
  __host__ __device__ static constexpr int midx(int m) { return STRESS ? (m - M_LAM) : (m - M_B1); }
  // byte offset of a box inside a plane-ring stage
  __host__ __device__ static constexpr int xhoff(int i) { return i * HSLOT; }
  __host__ __device__ static constexpr int h0off(int i) { return (NXH + i) * HSLOT; }
  __host__ __device__ static constexpr int poff(int i) { return (NXH + NH0) * HSLOT + i * PSLOT; }
  __host__ __device__ static constexpr int moff(int i) { return (NXH + NH0) * HSLOT + NPF * PSLOT + i * MSLOT; }
};

// Accessor of the generated expressions: xs[k] is the x-window stage of plane
// x + k - R, cs the plane-ring stage of plane x; hpos/ppos the thread's
// element offset inside a halo box / point box.  Every read is one shared
// load at a compile-time offset from one of these bases.
template <int R, typename S, int HET, bool STRESS>
struct TiledAcc {
  typedef TiledCfg<R, S, HET, STRESS> G;
  typedef typename Storage<S>::C C;
  const unsigned char *xs[2 * R + 1];
  const unsigned char *cs;
  const float *inv;
  int hpos, ppos, bpos;
  __device__ __forceinline__ C operator()(int f, int dx, int dy, int dz) const {
    const int off = dy * G::HW + dz;
    if (G::role(f) == 0) {
      if (G::SPLIT && dy == 0 && dz == 0) {
        const S *b = (const S *)(xs[dx + R] + G::xidx(f) * G::XSLOT);
        return (C)Storage<S>::load(b[ppos], inv[f]);
      }
      if (G::SPLIT) {
        const S *b = (const S *)(cs + G::xhoff(G::xhidx(f)));
        return (C)Storage<S>::load(b[hpos + off], inv[f]);
      }
      const S *b = (const S *)(xs[dx + R] + G::xidx(f) * G::XSLOT);
      return (C)Storage<S>::load(b[hpos + off], inv[f]);
    }
    if (G::role(f) == 1) {
      const S *b = (const S *)(cs + G::h0off(G::h0idx(f)));
      return (C)Storage<S>::load(b[hpos + off], inv[f]);
    }
    const S *b = (const S *)(cs + G::poff(G::pidx(f)));
    return (C)Storage<S>::load(b[ppos], inv[f]);
  }
  __device__ __forceinline__ C m(int i) const {
    if constexpr (G::NBX != 0) {
      // beta1..3 = (beta + beta at x+1 / y+1 / z+1) * 0.5f, as media_avg_kernel
      const float *b = (const float *)(xs[R] + G::NXF * G::XSLOT);
      const float b0 = b[bpos];
      float b1;
      if (i == M_B1) b1 = ((const float *)(xs[R + 1] + G::NXF * G::XSLOT))[bpos];
      else if (i == M_B2) b1 = b[bpos + G::BW];
      else b1 = b[bpos + 1];
      return (C)((b0 + b1) * 0.5f);
    }
    const float *b = (const float *)(cs + G::moff(G::midx(i)));
    return (C)b[ppos];
  }
};

// Accessor of the paired evaluation: the same reads as TiledAcc for the two
// points (z, z + 1) of the thread, as one register pair.  hpos, ppos and bpos
// are even, so a read at an even z offset is one vector load of both values
// and a read at an odd offset two scalar loads.
template <int R, typename S, int HET, bool STRESS>
struct TiledAcc2 {
  typedef TiledCfg<R, S, HET, STRESS> G;
  const unsigned char *xs[2 * R + 1];
  const unsigned char *cs;
  const float *inv;
  F2 nz;   // -0.0 pair from a kernel argument (see ofd_f32x2.cuh)
  int hpos, ppos, bpos;
  __device__ __forceinline__ F2 operator()(int f, int dx, int dy, int dz) const {
    const S *b;
    int pos;
    if (G::role(f) == 0 && G::SPLIT && dy == 0 && dz == 0) {
      b = (const S *)(xs[dx + R] + G::xidx(f) * G::XSLOT);
      pos = ppos;
    } else if (G::role(f) == 0 && G::SPLIT) {
      b = (const S *)(cs + G::xhoff(G::xhidx(f)));
      pos = hpos + dy * G::HW + dz;
    } else if (G::role(f) == 0) {
      b = (const S *)(xs[dx + R] + G::xidx(f) * G::XSLOT);
      pos = hpos + dy * G::HW + dz;
    } else if (G::role(f) == 1) {
      b = (const S *)(cs + G::h0off(G::h0idx(f)));
      pos = hpos + dy * G::HW + dz;
    } else {
      b = (const S *)(cs + G::poff(G::pidx(f)));
      pos = ppos;
    }
    if ((dz & 1) == 0) return PairLoad<S, true>::ld(b + pos, inv[f], nz);
    return PairLoad<S, false>::ld(b + pos, inv[f], nz);
  }
  __device__ __forceinline__ F2 m(int i) const {
    if constexpr (G::NBX != 0) {
      // beta1..3 = (beta + beta at x+1 / y+1 / z+1) * 0.5f, as media_avg_kernel
      const float *b = (const float *)(xs[R] + G::NXF * G::XSLOT);
      const F2 b0 = PairLoad<float, true>::ld(b + bpos, 1.f, nz);
      F2 b1;
      if (i == M_B1) b1 = PairLoad<float, true>::ld((const float *)(xs[R + 1] + G::NXF * G::XSLOT) + bpos, 1.f, nz);
      else if (i == M_B2) b1 = PairLoad<float, true>::ld(b + bpos + G::BW, 1.f, nz);
      else b1 = PairLoad<float, false>::ld(b + bpos + 1, 1.f, nz);
      // the sum is rounded, then halved (a product of a sum: nothing to fuse)
      return (b0 + b1) * f2(0.5f);
    }
    const float *b = (const float *)(cs + G::moff(G::midx(i)));
    return PairLoad<float, true>::ld(b + ppos, 1.f, nz);
  }
};

// Launch shape of a tiled sweep: 32 threads per consumer warp plus the
// producer warp, and the resident CTAs per SM the register budget is sized
// for.  Space order >= 6 with FP32 storage keeps one CTA per SM (its rings
// fill shared memory), so ptxas may use the whole register file rather than
// spill; lower orders and paired 16-bit storage keep two CTAs per SM.
template <int R, typename S, int HET> struct TiledLaunch {
  static constexpr int ZW = PairMode<S, HET>::v ? 1 : row_warps(R);
  static constexpr int THREADS = 32 * (tile_rows(R) * ZW + 1);
  static constexpr int MIN_BLOCKS = R >= 3 ? ((PairMode<S, HET>::v && sizeof(S) == 2) ? 2 : 1) : 2;
};

// The literal table of a heterogeneous expression held as its few distinct
// values (KMap): v[u] is the value of every literal with index map u.  The
// generated code indexes K with constants, so each K[i] becomes a register.
template <int R, bool STRESS>
struct KRegs {
  float v[KMap<R, STRESS>::NU];
  __device__ __forceinline__ float operator[](int i) const { return v[KMap<R, STRESS>::at(i)]; }
};

// The same for the paired evaluation: each distinct value as a pair {K, K},
// with the -0 addend of the products (ofd_f32x2.cuh).
template <int R, bool STRESS>
struct KRegs2 {
  F2 v[KMap<R, STRESS>::NU];
  F2 nz;
  __device__ __forceinline__ KF2 operator[](int i) const { return KF2{v[KMap<R, STRESS>::at(i)], nz}; }
};

// Literal table of the paired evaluation read from memory (tables that do not
// follow KMap, e.g. grids with different spacings along the axes).
struct KPairPtr {
  const float *k;
  F2 nz;
  __device__ __forceinline__ KF2 operator[](int i) const { return KF2{f2(k[i]), nz}; }
};

// One CTA's work: tile `tile` (z fastest) of the 64 x 8 tiling, x chunk
// `chunk`.  a and p live in kernel parameters (single-handle launch) or in a
// device table (grouped launch); K is the literal table (a pointer, or
// KRegs).
template <int R, typename S, int HET, bool STRESS, class KT>
__device__ __forceinline__ void sweep_tile(const SweepArgs<S> &a, const TiledParams &p, int tile, int chunk,
                                           const KT &K, unsigned char *smem_raw) {
  typedef TiledCfg<R, S, HET, STRESS> G;
  typedef typename Storage<S>::C C;
  unsigned char *smem = (unsigned char *)(((uintptr_t)smem_raw + 127) & ~(uintptr_t)127);
  unsigned char *xring = smem;
  unsigned char *cring = smem + G::XRING;
  uint64_t *xbar = (uint64_t *)(smem + G::XRING + G::CRING);   // x-window slots filled
  uint64_t *cbar = xbar + G::NSH;                                // plane-ring slots filled
  uint64_t *xemp = cbar + G::NSC;                                // x-window slots released
  uint64_t *cemp = xemp + G::NSH;                                // plane-ring slots released
  __shared__ int abort_flag;

  const Geom &g = a.g;
  constexpr int TY = G::TY;
  const int tz = tile % p.ntz, ty = tile / p.ntz;
  const int z0 = g.m + tz * TZ, y0 = g.m + ty * TY;
  const int xb = g.m + chunk * p.chunk;
  const int xe = min(xb + p.chunk, g.n1 - g.m);
  if (xb >= xe) return;
  const int hq0 = xb - R;          // plane of x-window ring q = 0
  const int hlast = xe - 1 + R;    // last x-window plane needed
  const int tid = threadIdx.x;
  const int zc = p.zcoord0 + (z0 - g.m);

  auto issue_x = [&](int plane) {
    const int slot = (plane - hq0) % G::NSH;
    uint64_t *bar = &xbar[slot];
    mbar_expect_tx(bar, G::XBYTES);
    unsigned char *st = xring + slot * G::XSTAGE;
#pragma unroll
    for (int i = 0; i < G::NXF; ++i) {
      if constexpr (G::SPLIT) tma_load_3d(st + i * G::XSLOT, &p.xpmap[i], bar, zc, y0, plane);
      else tma_load_3d(st + i * G::XSLOT, &p.hmap[i], bar, zc - G::ZH, y0 - R, plane);
    }
    if constexpr (G::NBX != 0) tma_load_3d(st + G::NXF * G::XSLOT, &p.bmap, bar, zc, y0, plane);
  };
  auto issue_c = [&](int plane) {
    const int slot = (plane - xb) % G::NSC;
    uint64_t *bar = &cbar[slot];
    mbar_expect_tx(bar, G::CBYTES);
    unsigned char *st = cring + slot * G::CSTAGE;
    // current-plane halo boxes of the X arrays read with y/z neighbours
    // (split staging): stress U V W = hmap[0..2], velocity Txy Txz = hmap[1..2]
#pragma unroll
    for (int i = 0; i < G::NXH; ++i)
      tma_load_3d(st + G::xhoff(i), &p.hmap[STRESS ? i : i + 1], bar, zc - G::ZH, y0 - R, plane);
#pragma unroll
    for (int i = 0; i < G::NH0; ++i) tma_load_3d(st + G::h0off(i), &p.hmap[G::NXF + i], bar, zc - G::ZH, y0 - R, plane);
#pragma unroll
    for (int i = 0; i < G::NPF; ++i) tma_load_3d(st + G::poff(i), &p.pmap[i], bar, zc, y0, plane);
#pragma unroll
    for (int i = 0; i < G::NMF; ++i) tma_load_3d(st + G::moff(i), &p.mmap[i], bar, zc, y0, plane);
  };

  // Warp specialisation: warps 0..NCW-1 compute (ZW per tile row); warp NCW is
  // the producer, whose lane 0 issues every TMA load.  A slot is refilled
  // once all consumer warps have released it (empty barrier, NCW arrivals),
  // so consumers never wait on each other, only on their data.
  const int warp = tid >> 5, lane = tid & 31;
  if (tid == 0) {
    abort_flag = 0;
    for (int i = 0; i < G::NSH; ++i) { mbar_init(&xbar[i], 1); mbar_init(&xemp[i], G::NCW); }
    for (int i = 0; i < G::NSC; ++i) { mbar_init(&cbar[i], 1); mbar_init(&cemp[i], G::NCW); }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();

  int hissued = hq0 - 1, pissued = xb - 1;   // last plane issued (producer)
  if (warp == G::NCW) {
    if (lane == 0) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      for (int pl = hq0; pl <= hlast && pl < hq0 + G::NSH; ++pl) { issue_x(pl); hissued = pl; }
      for (int pl = xb; pl < xe && pl < xb + G::NSC; ++pl) { issue_c(pl); pissued = pl; }
      // then in the order the consumers need them: x-window plane P at
      // iteration P - R, plane-ring plane P at iteration P
      while (hissued < hlast || pissued < xe - 1) {
        const bool take_x = hissued < hlast && (pissued >= xe - 1 || hissued + 1 - R <= pissued + 1);
        if (take_x) {
          const int q = hissued + 1 - hq0;
          if (!mbar_wait_or_abort(&xemp[q % G::NSH], (unsigned)((q / G::NSH - 1) & 1), &abort_flag, p.wait_ns)) break;
          asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
          issue_x(hissued + 1);
          ++hissued;
        } else {
          const int q = pissued + 1 - xb;
          if (!mbar_wait_or_abort(&cemp[q % G::NSC], (unsigned)((q / G::NSC - 1) & 1), &abort_flag, p.wait_ns)) break;
          asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
          issue_c(pissued + 1);
          ++pissued;
        }
      }
      if (hissued < hlast || pissued < xe - 1) {
        atomicExch(p.err, 1);
        abort_flag = 1;
      }
    }
  } else {
    const int yl = warp / G::ZW, zpart = warp % G::ZW;
    const int y = y0 + yl;
    const long step = a.sr ? *a.step : 0;   // rounding hash of 16-bit stores
    int hwaited = hq0 - 1;   // last x-window plane waited for
    for (int x = xb; x < xe; ++x) {
      bool ok = true;
      for (int pl = hwaited + 1; pl <= x + R && ok; ++pl) {
        const int q = pl - hq0;
        if (!mbar_wait_or_abort(&xbar[q % G::NSH], (unsigned)((q / G::NSH) & 1), &abort_flag, p.wait_ns)) ok = false;
        else hwaited = pl;
      }
      if (ok) {
        const int q = x - xb;
        if (!mbar_wait_or_abort(&cbar[q % G::NSC], (unsigned)((q / G::NSC) & 1), &abort_flag, p.wait_ns)) ok = false;
      }
      // leave as a whole warp (the release below is warp-synchronous)
      if (!__all_sync(0xffffffffu, ok)) {
        if (lane == 0) {
          atomicExch(p.err, 1);
          abort_flag = 1;
        }
        break;
      }
      if constexpr (G::PAIR) {
        // two adjacent z points per lane (z0 + 2 lane, + 1), f32x2 arithmetic
        TiledAcc2<R, S, HET, STRESS> A;
#pragma unroll
        for (int k = 0; k < 2 * R + 1; ++k) A.xs[k] = xring + ((x + k - R - hq0) % G::NSH) * G::XSTAGE;
        A.cs = cring + ((x - xb) % G::NSC) * G::CSTAGE;
        A.inv = a.inv;
        A.nz = f2(a.nz);
        const int zl = 2 * lane;
        const int z = z0 + zl;
        A.hpos = (yl + R) * G::HW + zl + G::ZH;
        A.ppos = yl * TZ + zl;
        A.bpos = yl * G::BW + zl;
        const long o = (long)x * g.plane + (long)y * g.P + z;
        const bool in0 = (z < g.n3 - g.m) && (y < g.n2 - g.m);
        const bool in1 = in0 && (z + 1 < g.n3 - g.m);
        if (STRESS) {
          F2 out[6];
          GenSweep<R, HET>::template stress<F2>(A, K, out);
          if (in0) {
#pragma unroll
            for (int i = 0; i < 6; ++i)
              PairStore<S>::st(a.out[F_TXX + i] + o, out[i], a.sc[F_TXX + i], in1, a.sr, o, F_TXX + i, step);
          }
        } else {
          F2 out[3];
          GenSweep<R, HET>::template velocity<F2>(A, K, out);
          if (in0) {
#pragma unroll
            for (int i = 0; i < 3; ++i)
              PairStore<S>::st(a.out[F_U + i] + o, out[i], a.sc[F_U + i], in1, a.sr, o, F_U + i, step);
          }
        }
      } else {
        TiledAcc<R, S, HET, STRESS> A;
#pragma unroll
        for (int k = 0; k < 2 * R + 1; ++k) A.xs[k] = xring + ((x + k - R - hq0) % G::NSH) * G::XSTAGE;
        A.cs = cring + ((x - xb) % G::NSC) * G::CSTAGE;
        A.inv = a.inv;
#pragma unroll
        for (int half = 0; half < 2 / G::ZW; ++half) {
          const int zl = lane + 32 * (zpart + half);
          const int z = z0 + zl;
          A.hpos = (yl + R) * G::HW + zl + G::ZH;
          A.ppos = yl * TZ + zl;
          A.bpos = yl * G::BW + zl;
          const long o = (long)x * g.plane + (long)y * g.P + z;
          const bool inside = (z < g.n3 - g.m) && (y < g.n2 - g.m);
          if (STRESS) {
            C out[6];
            GenSweep<R, HET>::template stress<C>(A, K, out);
            if (inside) {
#pragma unroll
              for (int i = 0; i < 6; ++i)
                a.out[F_TXX + i][o] =
                    SweepStore<S>::st(out[i], a.sc[F_TXX + i], a.sr, a.sr ? sr_hash(o, F_TXX + i, step) : 0u);
            }
          } else {
            C out[3];
            GenSweep<R, HET>::template velocity<C>(A, K, out);
            if (inside) {
#pragma unroll
              for (int i = 0; i < 3; ++i)
                a.out[F_U + i][o] =
                    SweepStore<S>::st(out[i], a.sc[F_U + i], a.sr, a.sr ? sr_hash(o, F_U + i, step) : 0u);
            }
          }
        }
      }
      // this warp is done with x-window plane x - R and plane-ring plane x
      __syncwarp();
      if (lane == 0) {
        mbar_arrive(&xemp[(x - R - hq0) % G::NSH]);
        mbar_arrive(&cemp[(x - xb) % G::NSC]);
      }
    }
  }
  __syncthreads();
  if (abort_flag && warp == G::NCW && lane == 0) {
    // drain: wait (bounded) for the last load issued into every slot, so that
    // no copy is still writing this CTA's shared memory when it exits
    for (int pl = hissued; pl > hissued - G::NSH && pl >= hq0; --pl) {
      const int q = pl - hq0;
      mbar_wait(&xbar[q % G::NSH], (unsigned)((q / G::NSH) & 1));
    }
    for (int pl = pissued; pl > pissued - G::NSC && pl >= xb; --pl) {
      const int q = pl - xb;
      mbar_wait(&cbar[q % G::NSC], (unsigned)((q / G::NSC) & 1));
    }
  }
}

// Single-handle sweep.  KD (paired evaluation only): the handle's literal
// table follows KMap, and each thread holds its distinct values as register
// pairs; otherwise pairs are formed from the table at every use.
template <int R, typename S, int HET, bool STRESS, bool KD = false>
__global__ void __launch_bounds__(TiledLaunch<R, S, HET>::THREADS, TiledLaunch<R, S, HET>::MIN_BLOCKS)
sweep_tiled(const __grid_constant__ SweepArgs<S> a, const __grid_constant__ TiledParams p) {
  extern __shared__ unsigned char smem_raw[];
  if constexpr (PairMode<S, HET>::v) {
    if constexpr (KD) {
      KRegs2<R, STRESS> kr;
#pragma unroll
      for (int i = 0; i < KMap<R, STRESS>::NK; ++i) kr.v[KMap<R, STRESS>::at(i)] = f2(a.K[i]);
      kr.nz = f2(a.nz);
      sweep_tile<R, S, HET, STRESS>(a, p, blockIdx.x, blockIdx.y, kr, smem_raw);
    } else {
      sweep_tile<R, S, HET, STRESS>(a, p, blockIdx.x, blockIdx.y, KPairPtr{a.K, f2(a.nz)}, smem_raw);
    }
  } else {
    sweep_tile<R, S, HET, STRESS>(a, p, blockIdx.x, blockIdx.y, (const float *)a.K, smem_raw);
  }
}

// One member of a grouped sweep launch: its arguments, descriptors and the
// range of the launch's CTAs that work on it.
template <typename S>
struct GroupSweep {
  TiledParams p;        // first: CUtensorMap members need 64-byte alignment
  SweepArgs<S> a;
  int cta_begin;        // first CTA of this member
  int tiles;            // tiles of this member (CTAs = tiles x chunks)
};

// Grouped sweep: CTA blockIdx.x works on the member whose range holds it
// (binary search over the table, sorted by cta_begin).  The descriptors were
// copied to global memory by the host before the launch; the producer lane
// orders them for the tensor-map proxy before its first load.  KD: the
// members' literal tables follow KMap (checked on the host), and each thread
// holds the distinct values in registers instead of reading the table from
// global memory at every use.
template <int R, typename S, int HET, bool STRESS, bool KD>
__global__ void __launch_bounds__(TiledLaunch<R, S, HET>::THREADS, TiledLaunch<R, S, HET>::MIN_BLOCKS)
sweep_tiled_group(const GroupSweep<S> *__restrict__ tab, int n) {
  extern __shared__ unsigned char smem_raw[];
  __shared__ int s_member;
  typedef TiledCfg<R, S, HET, STRESS> G;
  if (threadIdx.x == 0) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (tab[mid].cta_begin <= (int)blockIdx.x) lo = mid;
      else hi = mid - 1;
    }
    s_member = lo;
  }
  __syncthreads();
  const GroupSweep<S> &e = tab[s_member];
  // descriptors must sit on 64-byte boundaries (the host aligns the table);
  // a misplaced table is reported, never used
  if (((uintptr_t)&e.p) & 63) {
    if (threadIdx.x == 0) atomicExch(e.p.err, 4);
    return;
  }
  if (threadIdx.x == 32 * G::NCW) {
    const int nmaps = G::NXF + G::NH0;
#pragma unroll 1
    for (int i = 0; i < nmaps; ++i)
      asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(&e.p.hmap[i]) : "memory");
#pragma unroll 1
    for (int i = 0; i < G::NPF; ++i)
      asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(&e.p.pmap[i]) : "memory");
#pragma unroll 1
    for (int i = 0; i < G::NMF; ++i)
      asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(&e.p.mmap[i]) : "memory");
    if (G::NBX) asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(&e.p.bmap) : "memory");
    if (G::SPLIT) {
#pragma unroll 1
      for (int i = 0; i < G::NXF; ++i)
        asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(&e.p.xpmap[i]) : "memory");
    }
  }
  const int local = (int)blockIdx.x - e.cta_begin;
  if constexpr (KD && PairMode<S, HET>::v) {
    KRegs2<R, STRESS> kr;
#pragma unroll
    for (int i = 0; i < KMap<R, STRESS>::NK; ++i) kr.v[KMap<R, STRESS>::at(i)] = f2(e.a.K[i]);
    kr.nz = f2(e.a.nz);
    sweep_tile<R, S, HET, STRESS>(e.a, e.p, local % e.tiles, local / e.tiles, kr, smem_raw);
  } else if constexpr (KD) {
    KRegs<R, STRESS> kr;
#pragma unroll
    for (int i = 0; i < KMap<R, STRESS>::NK; ++i) kr.v[KMap<R, STRESS>::at(i)] = e.a.K[i];
    sweep_tile<R, S, HET, STRESS>(e.a, e.p, local % e.tiles, local / e.tiles, kr, smem_raw);
  } else if constexpr (PairMode<S, HET>::v) {
    sweep_tile<R, S, HET, STRESS>(e.a, e.p, local % e.tiles, local / e.tiles, KPairPtr{e.a.K, f2(e.a.nz)},
                                  smem_raw);
  } else {
    sweep_tile<R, S, HET, STRESS>(e.a, e.p, local % e.tiles, local / e.tiles, (const float *)e.a.K, smem_raw);
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
  if (g.n3 - 2 * g.m < TZ / 2 || g.n2 - 2 * g.m < tile_rows(R)) return false;
  return tiled_fits<R, S, 1, true>() && tiled_fits<R, S, 1, false>() && tiled_fits<R, S, 0, true>() &&
         tiled_fits<R, S, 0, false>();
}

// Descriptors and tiling of one sweep launch; returns the CTA grid (tiles,
// chunks).  chunk_planes > 0 forces the x chunk length (grouped launches),
// else the chunking aims at ~8 waves (x ctx.waves) of 152 SMs.
template <int R, typename S, int HET, bool STRESS>
void tiled_params(const SweepArgs<S> &a, const TiledCtx &ctx, int t0, int chunk_planes, TiledParams &p,
                  int *tiles_out, int *chunks_out) {
  typedef TiledCfg<R, S, HET, STRESS> G;
  const TmaMaps *mp = ctx.maps;
  const Geom &g = a.g;
  const int t1 = 1 - t0;
  if (STRESS) {
    for (int i = 0; i < 3; ++i) p.hmap[i] = mp->halo[F_U + i][t0];
    for (int i = 0; i < 3; ++i) p.xpmap[i] = mp->point[F_U + i][t0];
    for (int i = 0; i < 6; ++i) p.pmap[i] = mp->point[F_TXX + i][t0];
    for (int i = 0; i < 5; ++i) p.mmap[i] = mp->media[M_LAM + i];
  } else {
    // x-window arrays first (Txx Txy Txz), then plane-halo arrays (Tyy Tyz Tzz)
    const int order[6] = {F_TXX, F_TXY, F_TXZ, F_TYY, F_TYZ, F_TZZ};
    for (int i = 0; i < 6; ++i) p.hmap[i] = mp->halo[order[i]][t1];
    for (int i = 0; i < 3; ++i) p.xpmap[i] = mp->point[order[i]][t1];
    for (int i = 0; i < 3; ++i) p.pmap[i] = mp->point[F_U + i][t0];
    if (G::NBX) p.bmap = mp->beta;
  }
  p.err = ctx.err;
  p.wait_ns = ctx.wait_ns;
  p.zcoord0 = ctx.z0 + g.m;
  const int nx = g.n1 - 2 * g.m, ny = g.n2 - 2 * g.m, nz = g.n3 - 2 * g.m;
  p.ntz = (nz + TZ - 1) / TZ;
  p.nty = (ny + G::TY - 1) / G::TY;
  const long tiles = (long)p.ntz * p.nty;
  // enough CTAs for ~8 waves (x ctx.waves) of 152 SMs at the resident count,
  // chunks >= 16 planes
  const int per_sm = (227 * 1024) / (G::SMEM + 1024) > 0 ? (227 * 1024) / (G::SMEM + 1024) : 1;
  long want = 152L * per_sm * 8 * (ctx.waves > 0 ? ctx.waves : 1);
  int chunks = (int)((want + tiles - 1) / tiles);
  if (chunks > nx / 16) chunks = nx / 16;
  if (chunks < 1) chunks = 1;
  p.chunk = (nx + chunks - 1) / chunks;
  if (chunk_planes > 0) p.chunk = chunk_planes < nx ? chunk_planes : nx;
  chunks = (nx + p.chunk - 1) / p.chunk;
  *tiles_out = (int)tiles;
  *chunks_out = chunks;
}

template <int R, typename S, int HET, bool STRESS>
void launch_tiled(const SweepArgs<S> &a, const TiledCtx &ctx, int t0, cudaStream_t st) {
  typedef TiledCfg<R, S, HET, STRESS> G;
  TiledParams p;
  int tiles, chunks;
  tiled_params<R, S, HET, STRESS>(a, ctx, t0, 0, p, &tiles, &chunks);
  const dim3 grid((unsigned)tiles, (unsigned)chunks);
  if (HET && ctx.kd[STRESS ? 1 : 0]) sweep_tiled<R, S, HET, STRESS, HET != 0><<<grid, G::THREADS, G::SMEM, st>>>(a, p);
  else sweep_tiled<R, S, HET, STRESS, false><<<grid, G::THREADS, G::SMEM, st>>>(a, p);
}

// Dynamic shared memory opt-in of both sweeps; called once per handle so that
// launches can later be captured in a CUDA graph.
template <int R, typename S, int HET>
void prepare_tiled() {
  if (tiled_fits<R, S, HET, true>()) {
    const int sm = TiledCfg<R, S, HET, true>::SMEM;
    cudaFuncSetAttribute(sweep_tiled<R, S, HET, true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
    cudaFuncSetAttribute(sweep_tiled_group<R, S, HET, true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
    if constexpr (HET) {
      cudaFuncSetAttribute(sweep_tiled<R, S, HET, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
      cudaFuncSetAttribute(sweep_tiled_group<R, S, HET, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
    }
  }
  if (tiled_fits<R, S, HET, false>()) {
    const int sm = TiledCfg<R, S, HET, false>::SMEM;
    cudaFuncSetAttribute(sweep_tiled<R, S, HET, false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
    cudaFuncSetAttribute(sweep_tiled_group<R, S, HET, false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
    if constexpr (HET) {
      cudaFuncSetAttribute(sweep_tiled<R, S, HET, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
      cudaFuncSetAttribute(sweep_tiled_group<R, S, HET, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
    }
  }
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
