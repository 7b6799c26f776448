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
};

}  // namespace ofd
