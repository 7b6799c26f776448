// Paired FP32 arithmetic for the tiled sweeps: two grid points per thread
// evaluated with Blackwell's packed f32x2 instructions, which round each half
// exactly like the scalar .rn instructions (IEEE round to nearest, subnormals
// kept; measured bit for bit against the scalar forms).  One instruction
// advances two points, which halves the FP32 issue slots of the update
// expressions while their results stay bit for bit those of the scalar
// evaluation (and therefore of the reference's C expression): every product
// and sum is rounded on its own, in the printed order.
//
// No contraction.  The assembler fuses an f32x2 multiply that feeds an f32x2
// add into one fused multiply-add even with explicit .rn rounding and
// --fmad=false (measured: about 4.5 % of acc + (k*a)*m results differ from the
// scalar evaluation by one ulp).  Every product of the update expression is
// therefore formed as fma.rn.f32x2(x, y, nz) with nz = -0.0 taken from a kernel
// argument: x*y + (-0) is exactly round(x*y) for every x*y (including a
// product of -0), and the assembler cannot fold an addend whose value it does
// not know, so the product stays rounded on its own before it is accumulated.
//
// F2 is a 64-bit register pair {lo, hi}; lo belongs to the thread's lower z
// point, hi to z + 1.
#pragma once
#include <cuda_fp16.h>
#include <cuda_bf16.h>
#include "ofd_common.cuh"

namespace ofd {

struct F2 {
  unsigned long long v;
};

__device__ __forceinline__ F2 f2(float lo, float hi) {
  F2 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r.v) : "f"(lo), "f"(hi));
  return r;
}
__device__ __forceinline__ F2 f2(float a) { return f2(a, a); }

__device__ __forceinline__ float f2_lo(F2 a) { return __uint_as_float((unsigned)(a.v & 0xffffffffULL)); }
__device__ __forceinline__ float f2_hi(F2 a) { return __uint_as_float((unsigned)(a.v >> 32)); }

__device__ __forceinline__ F2 operator*(F2 a, F2 b) {
  F2 r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
  return r;
}
__device__ __forceinline__ F2 operator+(F2 a, F2 b) {
  F2 r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
  return r;
}
__device__ __forceinline__ F2 operator-(F2 a, F2 b) {
  F2 r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
  return r;
}
// negation flips both sign bits (exact, as the scalar neg.f32)
__device__ __forceinline__ F2 operator-(F2 a) {
  F2 r;
  r.v = a.v ^ 0x8000000080000000ULL;
  return r;
}
__device__ __forceinline__ F2 fma2(F2 a, F2 b, F2 c) {
  F2 r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r.v) : "l"(a.v), "l"(b.v), "l"(c.v));
  return r;
}

// A literal of the update expression as a pair {K, K}, with the opaque -0
// addend (nz) of the products it starts.  The generated terms read
// K[i]*A(...)*A.m(...): the literal times an array value, then times a medium,
// left to right; each product is rounded on its own (fma2 with nz).
struct KF2 {
  F2 k, nz;
};
struct KProd {   // K[i]*A(...), rounded
  F2 v, nz;
};
__device__ __forceinline__ KF2 operator-(KF2 a) { return KF2{-a.k, a.nz}; }
__device__ __forceinline__ KProd operator*(KF2 k, F2 a) { return KProd{fma2(k.k, a, k.nz), k.nz}; }
__device__ __forceinline__ F2 operator*(KProd p, F2 m) { return fma2(p.v, m, p.nz); }
__device__ __forceinline__ F2 operator+(F2 a, KProd p) { return a + p.v; }
__device__ __forceinline__ F2 operator-(F2 a, KProd p) { return a - p.v; }

// Pair loads from shared memory of two consecutive elements p[0], p[1] of
// storage type S, converted to FP32 and unscaled (value = stored * inv, as
// Storage<S>::load, the product rounded on its own: fma2 with nz).  ALIGNED: p
// sits on a boundary of two elements, so one vector load fetches both.
template <typename S, bool ALIGNED> struct PairLoad;

template <bool ALIGNED> struct PairLoad<float, ALIGNED> {
  __device__ __forceinline__ static F2 ld(const float *p, float, F2) {
    if constexpr (ALIGNED) {
      const float2 v = *reinterpret_cast<const float2 *>(p);
      return f2(v.x, v.y);
    } else {
      return f2(p[0], p[1]);
    }
  }
};

template <bool ALIGNED> struct PairLoad<__half, ALIGNED> {
  __device__ __forceinline__ static F2 ld(const __half *p, float inv, F2 nz) {
    float a, b;
    if constexpr (ALIGNED) {
      const float2 v = __half22float2(*reinterpret_cast<const __half2 *>(p));
      a = v.x;
      b = v.y;
    } else {
      a = __half2float(p[0]);
      b = __half2float(p[1]);
    }
    return fma2(f2(a, b), f2(inv), nz);
  }
};

template <bool ALIGNED> struct PairLoad<__nv_bfloat16, ALIGNED> {
  __device__ __forceinline__ static F2 ld(const __nv_bfloat16 *p, float inv, F2 nz) {
    float a, b;
    if constexpr (ALIGNED) {
      const float2 v = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162 *>(p));
      a = v.x;
      b = v.y;
    } else {
      a = __bfloat162float(p[0]);
      b = __bfloat162float(p[1]);
    }
    return fma2(f2(a, b), f2(inv), nz);
  }
};

// Pair stores to global memory at an element offset of two-element alignment;
// both: both points lie inside the grid (else only the lower one is written).
// The stored value is value * sc rounded to S, as Storage<S>::store.
template <typename S> struct PairStore;

// sr: stochastic rounding of 16-bit stores (SweepStore) with the hash of
// element offsets o, o + 1 of field f at step.
template <> struct PairStore<float> {
  __device__ __forceinline__ static void st(float *p, F2 v, float, bool both, int, long, int, long) {
    if (both) *reinterpret_cast<float2 *>(p) = make_float2(f2_lo(v), f2_hi(v));
    else p[0] = f2_lo(v);
  }
};

template <> struct PairStore<__half> {
  __device__ __forceinline__ static void st(__half *p, F2 v, float sc, bool both, int sr, long o, int f, long step) {
    if (sr) {
      p[0] = SweepStore<__half>::st(f2_lo(v), sc, 1, sr_hash(o, f, step));
      if (both) p[1] = SweepStore<__half>::st(f2_hi(v), sc, 1, sr_hash(o + 1, f, step));
      return;
    }
    const F2 s = v * f2(sc);
    if (both) *reinterpret_cast<__half2 *>(p) = __floats2half2_rn(f2_lo(s), f2_hi(s));
    else p[0] = __float2half_rn(f2_lo(s));
  }
};

template <> struct PairStore<__nv_bfloat16> {
  __device__ __forceinline__ static void st(__nv_bfloat16 *p, F2 v, float sc, bool both, int sr, long o, int f,
                                            long step) {
    if (sr) {
      p[0] = SweepStore<__nv_bfloat16>::st(f2_lo(v), sc, 1, sr_hash(o, f, step));
      if (both) p[1] = SweepStore<__nv_bfloat16>::st(f2_hi(v), sc, 1, sr_hash(o + 1, f, step));
      return;
    }
    const F2 s = v * f2(sc);
    if (both) *reinterpret_cast<__nv_bfloat162 *>(p) = __floats2bfloat162_rn(f2_lo(s), f2_hi(s));
    else p[0] = __float2bfloat16_rn(f2_lo(s));
  }
};

}  // namespace ofd
