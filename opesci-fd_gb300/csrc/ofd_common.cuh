// Shared device-side types of the opesci-fd GB300 runtime: storage traits,
// padded field layout and the argument blocks of the sweep / ghost kernels.
//
// Layout in HBM (per field, two time levels): element (lvl, x, y, z) of a
// grid with dims (n1, n2, n3) lives at
//     base + lvl*level_stride + (x*n2 + y)*P + z0 + z
// x = dim1 (slowest), z = dim3 (contiguous), the axis names of the reference
// (regulargrid.py:466-496).  z0 shifts the first interior point z = m onto a
// 128-byte boundary and P rounds the row up to 128 bytes, so every warp-wide
// row access of the interior is sector aligned and 16-byte vector loads and
// TMA boxes start on aligned addresses.
#pragma once
#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <cuda_bf16.h>
#include <stdint.h>

#define OFD_MAX_K 160

namespace ofd {

enum { F_U = 0, F_V, F_W, F_TXX, F_TYY, F_TZZ, F_TXY, F_TYZ, F_TXZ, NF };
// media arrays: lambda, mu, the effective shear moduli, the averaged
// buoyancies and the buoyancy beta = 1/rho itself (from which the tiled
// velocity sweep forms beta1..3 on the fly)
enum { M_LAM = 0, M_MU, M_MU12, M_MU13, M_MU23, M_B1, M_B2, M_B3, M_BETA, NM };

// Storage traits: S is the stored type, C the arithmetic type.  16-bit
// storage keeps value*scale (scale a power of two, so scaling is exact).
template <typename S> struct Storage;
template <> struct Storage<float> {
  typedef float C;
  __device__ __forceinline__ static float load(float s, float) { return s; }
  __device__ __forceinline__ static float store(float v, float) { return v; }
};
template <> struct Storage<double> {
  typedef double C;
  __device__ __forceinline__ static double load(double s, float) { return s; }
  __device__ __forceinline__ static double store(double v, float) { return v; }
};
template <> struct Storage<__half> {
  typedef float C;
  __device__ __forceinline__ static float load(__half s, float inv) { return __half2float(s) * inv; }
  __device__ __forceinline__ static __half store(float v, float sc) { return __float2half_rn(v * sc); }
};
template <> struct Storage<__nv_bfloat16> {
  typedef float C;
  __device__ __forceinline__ static float load(__nv_bfloat16 s, float inv) { return __bfloat162float(s) * inv; }
  __device__ __forceinline__ static __nv_bfloat16 store(float v, float sc) { return __float2bfloat16_rn(v * sc); }
};

// Stochastic rounding of the 16-bit stores (optional, per handle).  A value
// v * scale between two adjacent 16-bit numbers lo < |v| < hi (same sign) is
// stored as hi with probability (|v| - lo) / (hi - lo), else lo, so the stored
// value is v in expectation: per-step increments smaller than half a unit in
// the last place, which round-to-nearest discards, accumulate on average.
// The random number is a deterministic hash of (element offset, field, step),
// so every kernel path (plain, tiled, grouped, persistent) stores the same
// bits.  The hash is the SplitMix64 output function (Steele, Lea and Flood,
// "Fast splittable pseudorandom number generators", OOPSLA 2014).
__device__ __forceinline__ unsigned sr_hash(long o, int f, long step) {
  unsigned long long x = (unsigned long long)o * 0x9E3779B97F4A7C15ULL;
  x ^= (unsigned long long)step * 0xC2B2AE3D27D4EB4FULL + ((unsigned long long)f << 58);
  x ^= x >> 30;
  x *= 0xBF58476D1CE4E5B9ULL;
  x ^= x >> 27;
  x *= 0x94D049BB133111EBULL;
  x ^= x >> 31;
  return (unsigned)x;
}

// lo: v rounded toward zero, hi: the next magnitude of the same sign
template <typename H, unsigned short (*TO_BITS)(H), H (*FROM_BITS)(unsigned short), H (*RZ)(float), float (*TO_F)(H)>
__device__ __forceinline__ H sr_round(float v, unsigned h, H (*RN)(float)) {
  const H r = RZ(v);
  const float rf = TO_F(r);
  const float d = fabsf(v - rf);              // exact: rf and v lie within one unit of each other
  if (d == 0.f || !isfinite(v)) return RN(v);
  const H nx = FROM_BITS((unsigned short)(TO_BITS(r) + 1));   // next magnitude, same sign
  const float step = fabsf(TO_F(nx) - rf);    // one unit in the last place (exact)
  const float u = (float)(h >> 8) * (1.0f / 16777216.0f);
  return (u * step < d) ? nx : r;             // u * step is exact (step a power of two)
}

__device__ __forceinline__ unsigned short half_bits(__half a) { return __half_as_ushort(a); }
__device__ __forceinline__ __half half_from(unsigned short b) { return __ushort_as_half(b); }
__device__ __forceinline__ __half half_rz(float v) { return __float2half_rz(v); }
__device__ __forceinline__ __half half_rn(float v) { return __float2half_rn(v); }
__device__ __forceinline__ float half_f(__half a) { return __half2float(a); }
__device__ __forceinline__ unsigned short bf16_bits(__nv_bfloat16 a) { return __bfloat16_as_ushort(a); }
__device__ __forceinline__ __nv_bfloat16 bf16_from(unsigned short b) { return __ushort_as_bfloat16(b); }
__device__ __forceinline__ __nv_bfloat16 bf16_rz(float v) { return __float2bfloat16_rz(v); }
__device__ __forceinline__ __nv_bfloat16 bf16_rn(float v) { return __float2bfloat16_rn(v); }
__device__ __forceinline__ float bf16_f(__nv_bfloat16 a) { return __bfloat162float(a); }

// Store of a sweep result: round to nearest, or stochastic (sr != 0) with the
// hash h; FP32 and FP64 storage ignore sr.
template <typename S> struct SweepStore {
  __device__ __forceinline__ static S st(typename Storage<S>::C v, float sc, int, unsigned) {
    return Storage<S>::store(v, sc);
  }
};
template <> struct SweepStore<__half> {
  __device__ __forceinline__ static __half st(float v, float sc, int sr, unsigned h) {
    if (!sr) return Storage<__half>::store(v, sc);
    return sr_round<__half, half_bits, half_from, half_rz, half_f>(v * sc, h, half_rn);
  }
};
template <> struct SweepStore<__nv_bfloat16> {
  __device__ __forceinline__ static __nv_bfloat16 st(float v, float sc, int sr, unsigned h) {
    if (!sr) return Storage<__nv_bfloat16>::store(v, sc);
    return sr_round<__nv_bfloat16, bf16_bits, bf16_from, bf16_rz, bf16_f>(v * sc, h, bf16_rn);
  }
};

struct Geom {
  int n1, n2, n3;      // dim1, dim2, dim3 (margins included)
  int m;               // margin = space_order / 2
  long P;              // row pitch (elements)
  long plane;          // n2 * P
  long level;          // elements between time levels of one field
};

// Arguments of one sweep launch.  Pointers are already offset by z0 and by the
// level they refer to, so element (x,y,z) is p[x*plane + y*P + z].
template <typename S> struct SweepArgs {
  Geom g;
  const S *in[NF];     // values read (stress sweep: all at t0; velocity sweep:
                       // velocities at t0, stresses at t1)
  S *out[NF];          // values written at t1
  const float *media[NM];
  float inv[NF];       // 1/scale per field (loads)
  float sc[NF];        // scale per field (stores)
  typename Storage<S>::C dt, ih1, ih2, ih3;
  typename Storage<S>::C c[4];
  int xchunk;          // planes per CTA along x
  int sr;              // 16-bit storage: stochastic rounding of the stores (SweepStore)
  const long *step;    // device step counter (the step of this sweep, for the rounding hash)
  float nz;            // -0.0f: the addend that keeps paired products unfused (ofd_f32x2.cuh)
  float K[OFD_MAX_K];  // literal table of the generated update expression
};

// Ghost-cell launch arguments: one level, per-face algorithm.
template <typename S> struct BcArgs {
  Geom g;
  S *f1[NF];           // level written (t1)
  const S *f0[NF];     // level t0 (stress recompute)
  const float *media[NM];
  float inv[NF], sc[NF];
  int face[6];         // ofd_face_bc per face x-,x+,y-,y+,z-,z+
  int recompute;       // Levander normal-stress recompute enabled
  int d;               // face normal axis of this phase (0..2)
  int sub;             // velocity: 0 = component along d, 1 = the other two
  typename Storage<S>::C dt, h[3];
  typename Storage<S>::C c4[2];  // 4th-order weights 9/8, -1/24
  // space order 4, Levander faces: evaluate the generated ghost expressions
  // (GenGhost4<het>, literals kg in device memory) instead of the restated
  // formulas
  int gen, het;
  const float *kg;
  // normal-stress recompute values precomputed for this step (stress ghosts
  // with gen): rc[((d * 2 + side) * 2 + q) * rcs + i1 * n2(d) + i2], q the
  // index of the recomputed normal stress among the two of face normal d;
  // nullptr: evaluate in place
  const float *rc;
  long rcs;
};

}  // namespace ofd
