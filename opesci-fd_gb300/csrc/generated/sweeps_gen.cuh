// GENERATED by opesci/templates/cuda_gen.py from the symbolic kernels of
// StaggeredGrid (expanded, constant-folded, media resolved); do not edit.
// Each function evaluates the reference generator's C expression of the
// update with its literals taken from the table K; up to space order 4
// the sums of the outputs are interleaved term by term (each chain in
// its printed order).
#pragma once
#include "ofd_common.cuh"

namespace ofd {

template <int R, int HET> struct GenSweep { static constexpr bool ok = false; };

template <> struct GenSweep<1, 0> {
  static constexpr bool ok = true;
  static constexpr int NK_STRESS = 30, NK_VELOCITY = 18;
  template <typename C, class Acc, class KT>
  __device__ __forceinline__ static void stress(const Acc &A, const KT &K, C out[6]) {
    C o0 = A(F_TXX, 0, 0, 0);
    C o1 = A(F_TYY, 0, 0, 0);
    C o2 = A(F_TZZ, 0, 0, 0);
    C o3 = A(F_TXY, 0, 0, 0);
    C o4 = A(F_TYZ, 0, 0, 0);
    C o5 = A(F_TXZ, 0, 0, 0);
    o0 = o0 - K[0]*A(F_U, -1, 0, 0);
    o1 = o1 - K[6]*A(F_U, -1, 0, 0);
    o2 = o2 - K[12]*A(F_U, -1, 0, 0);
    o3 = o3 + K[18]*A(F_U, 0, 1, 0);
    o4 = o4 + K[22]*A(F_V, 0, 0, 1);
    o5 = o5 + K[26]*A(F_U, 0, 0, 1);
    o0 = o0 + K[1]*A(F_U, 0, 0, 0);
    o1 = o1 + K[7]*A(F_U, 0, 0, 0);
    o2 = o2 + K[13]*A(F_U, 0, 0, 0);
    o3 = o3 - K[19]*A(F_U, 0, 0, 0);
    o4 = o4 - K[23]*A(F_V, 0, 0, 0);
    o5 = o5 - K[27]*A(F_U, 0, 0, 0);
    o0 = o0 - K[2]*A(F_V, 0, -1, 0);
    o1 = o1 - K[8]*A(F_V, 0, -1, 0);
    o2 = o2 - K[14]*A(F_V, 0, -1, 0);
    o3 = o3 + K[20]*A(F_V, 1, 0, 0);
    o4 = o4 + K[24]*A(F_W, 0, 1, 0);
    o5 = o5 + K[28]*A(F_W, 1, 0, 0);
    o0 = o0 + K[3]*A(F_V, 0, 0, 0);
    o1 = o1 + K[9]*A(F_V, 0, 0, 0);
    o2 = o2 + K[15]*A(F_V, 0, 0, 0);
    o3 = o3 - K[21]*A(F_V, 0, 0, 0);
    o4 = o4 - K[25]*A(F_W, 0, 0, 0);
    o5 = o5 - K[29]*A(F_W, 0, 0, 0);
    o0 = o0 - K[4]*A(F_W, 0, 0, -1);
    o1 = o1 - K[10]*A(F_W, 0, 0, -1);
    o2 = o2 - K[16]*A(F_W, 0, 0, -1);
    o0 = o0 + K[5]*A(F_W, 0, 0, 0);
    o1 = o1 + K[11]*A(F_W, 0, 0, 0);
    o2 = o2 + K[17]*A(F_W, 0, 0, 0);
    out[0] = o0;
    out[1] = o1;
    out[2] = o2;
    out[3] = o3;
    out[4] = o4;
    out[5] = o5;
  }
  template <typename C, class Acc, class KT>
  __device__ __forceinline__ static void velocity(const Acc &A, const KT &K, C out[3]) {
    C o0 = K[0]*A(F_TXX, 1, 0, 0);
    C o1 = -K[6]*A(F_TXY, -1, 0, 0);
    C o2 = -K[12]*A(F_TXZ, -1, 0, 0);
    o0 = o0 - K[1]*A(F_TXX, 0, 0, 0);
    o1 = o1 + K[7]*A(F_TXY, 0, 0, 0);
    o2 = o2 + K[13]*A(F_TXZ, 0, 0, 0);
    o0 = o0 - K[2]*A(F_TXY, 0, -1, 0);
    o1 = o1 + K[8]*A(F_TYY, 0, 1, 0);
    o2 = o2 - K[14]*A(F_TYZ, 0, -1, 0);
    o0 = o0 + K[3]*A(F_TXY, 0, 0, 0);
    o1 = o1 - K[9]*A(F_TYY, 0, 0, 0);
    o2 = o2 + K[15]*A(F_TYZ, 0, 0, 0);
    o0 = o0 - K[4]*A(F_TXZ, 0, 0, -1);
    o1 = o1 - K[10]*A(F_TYZ, 0, 0, -1);
    o2 = o2 + K[16]*A(F_TZZ, 0, 0, 1);
    o0 = o0 + K[5]*A(F_TXZ, 0, 0, 0);
    o1 = o1 + K[11]*A(F_TYZ, 0, 0, 0);
    o2 = o2 - K[17]*A(F_TZZ, 0, 0, 0);
    o0 = o0 + A(F_U, 0, 0, 0);
    o1 = o1 + A(F_V, 0, 0, 0);
    o2 = o2 + A(F_W, 0, 0, 0);
    out[0] = o0;
    out[1] = o1;
    out[2] = o2;
  }
};

template <> struct GenSweep<1, 1> {
  static constexpr bool ok = true;
  static constexpr int NK_STRESS = 36, NK_VELOCITY = 18;
  template <typename C, class Acc, class KT>
  __device__ __forceinline__ static void stress(const Acc &A, const KT &K, C out[6]) {
    C o0 = A(F_TXX, 0, 0, 0);
    C o1 = A(F_TYY, 0, 0, 0);
    C o2 = A(F_TZZ, 0, 0, 0);
    C o3 = A(F_TXY, 0, 0, 0);
    C o4 = A(F_TYZ, 0, 0, 0);
    C o5 = A(F_TXZ, 0, 0, 0);
    o0 = o0 - K[0]*A(F_U, -1, 0, 0)*A.m(M_LAM);
    o1 = o1 - K[8]*A(F_U, -1, 0, 0)*A.m(M_LAM);
    o2 = o2 - K[16]*A(F_U, -1, 0, 0)*A.m(M_LAM);
    o3 = o3 + K[24]*A(F_U, 0, 1, 0)*A.m(M_MU12);
    o4 = o4 + K[28]*A(F_V, 0, 0, 1)*A.m(M_MU23);
    o5 = o5 + K[32]*A(F_U, 0, 0, 1)*A.m(M_MU13);
    o0 = o0 - K[1]*A(F_U, -1, 0, 0)*A.m(M_MU);
    o1 = o1 + K[9]*A(F_U, 0, 0, 0)*A.m(M_LAM);
    o2 = o2 + K[17]*A(F_U, 0, 0, 0)*A.m(M_LAM);
    o3 = o3 - K[25]*A(F_U, 0, 0, 0)*A.m(M_MU12);
    o4 = o4 - K[29]*A(F_V, 0, 0, 0)*A.m(M_MU23);
    o5 = o5 - K[33]*A(F_U, 0, 0, 0)*A.m(M_MU13);
    o0 = o0 + K[2]*A(F_U, 0, 0, 0)*A.m(M_LAM);
    o1 = o1 - K[10]*A(F_V, 0, -1, 0)*A.m(M_LAM);
    o2 = o2 - K[18]*A(F_V, 0, -1, 0)*A.m(M_LAM);
    o3 = o3 + K[26]*A(F_V, 1, 0, 0)*A.m(M_MU12);
    o4 = o4 + K[30]*A(F_W, 0, 1, 0)*A.m(M_MU23);
    o5 = o5 + K[34]*A(F_W, 1, 0, 0)*A.m(M_MU13);
    o0 = o0 + K[3]*A(F_U, 0, 0, 0)*A.m(M_MU);
    o1 = o1 - K[11]*A(F_V, 0, -1, 0)*A.m(M_MU);
    o2 = o2 + K[19]*A(F_V, 0, 0, 0)*A.m(M_LAM);
    o3 = o3 - K[27]*A(F_V, 0, 0, 0)*A.m(M_MU12);
    o4 = o4 - K[31]*A(F_W, 0, 0, 0)*A.m(M_MU23);
    o5 = o5 - K[35]*A(F_W, 0, 0, 0)*A.m(M_MU13);
    o0 = o0 - K[4]*A(F_V, 0, -1, 0)*A.m(M_LAM);
    o1 = o1 + K[12]*A(F_V, 0, 0, 0)*A.m(M_LAM);
    o2 = o2 - K[20]*A(F_W, 0, 0, -1)*A.m(M_LAM);
    o0 = o0 + K[5]*A(F_V, 0, 0, 0)*A.m(M_LAM);
    o1 = o1 + K[13]*A(F_V, 0, 0, 0)*A.m(M_MU);
    o2 = o2 - K[21]*A(F_W, 0, 0, -1)*A.m(M_MU);
    o0 = o0 - K[6]*A(F_W, 0, 0, -1)*A.m(M_LAM);
    o1 = o1 - K[14]*A(F_W, 0, 0, -1)*A.m(M_LAM);
    o2 = o2 + K[22]*A(F_W, 0, 0, 0)*A.m(M_LAM);
    o0 = o0 + K[7]*A(F_W, 0, 0, 0)*A.m(M_LAM);
    o1 = o1 + K[15]*A(F_W, 0, 0, 0)*A.m(M_LAM);
    o2 = o2 + K[23]*A(F_W, 0, 0, 0)*A.m(M_MU);
    out[0] = o0;
    out[1] = o1;
    out[2] = o2;
    out[3] = o3;
    out[4] = o4;
    out[5] = o5;
  }
  template <typename C, class Acc, class KT>
  __device__ __forceinline__ static void velocity(const Acc &A, const KT &K, C out[3]) {
    C o0 = K[0]*A(F_TXX, 1, 0, 0)*A.m(M_B1);
    C o1 = -K[6]*A(F_TXY, -1, 0, 0)*A.m(M_B2);
    C o2 = -K[12]*A(F_TXZ, -1, 0, 0)*A.m(M_B3);
    o0 = o0 - K[1]*A(F_TXX, 0, 0, 0)*A.m(M_B1);
    o1 = o1 + K[7]*A(F_TXY, 0, 0, 0)*A.m(M_B2);
    o2 = o2 + K[13]*A(F_TXZ, 0, 0, 0)*A.m(M_B3);
    o0 = o0 - K[2]*A(F_TXY, 0, -1, 0)*A.m(M_B1);
    o1 = o1 + K[8]*A(F_TYY, 0, 1, 0)*A.m(M_B2);
    o2 = o2 - K[14]*A(F_TYZ, 0, -1, 0)*A.m(M_B3);
    o0 = o0 + K[3]*A(F_TXY, 0, 0, 0)*A.m(M_B1);
    o1 = o1 - K[9]*A(F_TYY, 0, 0, 0)*A.m(M_B2);
    o2 = o2 + K[15]*A(F_TYZ, 0, 0, 0)*A.m(M_B3);
    o0 = o0 - K[4]*A(F_TXZ, 0, 0, -1)*A.m(M_B1);
    o1 = o1 - K[10]*A(F_TYZ, 0, 0, -1)*A.m(M_B2);
    o2 = o2 + K[16]*A(F_TZZ, 0, 0, 1)*A.m(M_B3);
    o0 = o0 + K[5]*A(F_TXZ, 0, 0, 0)*A.m(M_B1);
    o1 = o1 + K[11]*A(F_TYZ, 0, 0, 0)*A.m(M_B2);
    o2 = o2 - K[17]*A(F_TZZ, 0, 0, 0)*A.m(M_B3);
    o0 = o0 + A(F_U, 0, 0, 0);
    o1 = o1 + A(F_V, 0, 0, 0);
    o2 = o2 + A(F_W, 0, 0, 0);
    out[0] = o0;
    out[1] = o1;
    out[2] = o2;
  }
};

template <> struct GenSweep<2, 0> {
  static constexpr bool ok = true;
  static constexpr int NK_STRESS = 60, NK_VELOCITY = 36;
  template <typename C, class Acc, class KT>
  __device__ __forceinline__ static void stress(const Acc &A, const KT &K, C out[6]) {
    C o0 = A(F_TXX, 0, 0, 0);
    C o1 = A(F_TYY, 0, 0, 0);
    C o2 = A(F_TZZ, 0, 0, 0);
    C o3 = A(F_TXY, 0, 0, 0);
    C o4 = A(F_TYZ, 0, 0, 0);
    C o5 = A(F_TXZ, 0, 0, 0);
    o0 = o0 - K[0]*A(F_U, 1, 0, 0);
    o1 = o1 - K[12]*A(F_U, 1, 0, 0);
    o2 = o2 - K[24]*A(F_U, 1, 0, 0);
    o3 = o3 + K[36]*A(F_U, 0, 1, 0);
    o4 = o4 + K[44]*A(F_V, 0, 0, 1);
    o5 = o5 + K[52]*A(F_U, 0, 0, 1);
    o0 = o0 - K[1]*A(F_U, -1, 0, 0);
    o1 = o1 - K[13]*A(F_U, -1, 0, 0);
    o2 = o2 - K[25]*A(F_U, -1, 0, 0);
    o3 = o3 - K[37]*A(F_U, 0, 2, 0);
    o4 = o4 - K[45]*A(F_V, 0, 0, 2);
    o5 = o5 - K[53]*A(F_U, 0, 0, 2);
    o0 = o0 + K[2]*A(F_U, -2, 0, 0);
    o1 = o1 + K[14]*A(F_U, -2, 0, 0);
    o2 = o2 + K[26]*A(F_U, -2, 0, 0);
    o3 = o3 + K[38]*A(F_U, 0, -1, 0);
    o4 = o4 + K[46]*A(F_V, 0, 0, -1);
    o5 = o5 + K[54]*A(F_U, 0, 0, -1);
    o0 = o0 + K[3]*A(F_U, 0, 0, 0);
    o1 = o1 + K[15]*A(F_U, 0, 0, 0);
    o2 = o2 + K[27]*A(F_U, 0, 0, 0);
    o3 = o3 - K[39]*A(F_U, 0, 0, 0);
    o4 = o4 - K[47]*A(F_V, 0, 0, 0);
    o5 = o5 - K[55]*A(F_U, 0, 0, 0);
    o0 = o0 - K[4]*A(F_V, 0, 1, 0);
    o1 = o1 - K[16]*A(F_V, 0, 1, 0);
    o2 = o2 - K[28]*A(F_V, 0, 1, 0);
    o3 = o3 + K[40]*A(F_V, 1, 0, 0);
    o4 = o4 + K[48]*A(F_W, 0, 1, 0);
    o5 = o5 + K[56]*A(F_W, 1, 0, 0);
    o0 = o0 - K[5]*A(F_V, 0, -1, 0);
    o1 = o1 - K[17]*A(F_V, 0, -1, 0);
    o2 = o2 - K[29]*A(F_V, 0, -1, 0);
    o3 = o3 - K[41]*A(F_V, 2, 0, 0);
    o4 = o4 - K[49]*A(F_W, 0, 2, 0);
    o5 = o5 - K[57]*A(F_W, 2, 0, 0);
    o0 = o0 + K[6]*A(F_V, 0, -2, 0);
    o1 = o1 + K[18]*A(F_V, 0, -2, 0);
    o2 = o2 + K[30]*A(F_V, 0, -2, 0);
    o3 = o3 + K[42]*A(F_V, -1, 0, 0);
    o4 = o4 + K[50]*A(F_W, 0, -1, 0);
    o5 = o5 + K[58]*A(F_W, -1, 0, 0);
    o0 = o0 + K[7]*A(F_V, 0, 0, 0);
    o1 = o1 + K[19]*A(F_V, 0, 0, 0);
    o2 = o2 + K[31]*A(F_V, 0, 0, 0);
    o3 = o3 - K[43]*A(F_V, 0, 0, 0);
    o4 = o4 - K[51]*A(F_W, 0, 0, 0);
    o5 = o5 - K[59]*A(F_W, 0, 0, 0);
    o0 = o0 - K[8]*A(F_W, 0, 0, 1);
    o1 = o1 - K[20]*A(F_W, 0, 0, 1);
    o2 = o2 - K[32]*A(F_W, 0, 0, 1);
    o0 = o0 - K[9]*A(F_W, 0, 0, -1);
    o1 = o1 - K[21]*A(F_W, 0, 0, -1);
    o2 = o2 - K[33]*A(F_W, 0, 0, -1);
    o0 = o0 + K[10]*A(F_W, 0, 0, -2);
    o1 = o1 + K[22]*A(F_W, 0, 0, -2);
    o2 = o2 + K[34]*A(F_W, 0, 0, -2);
    o0 = o0 + K[11]*A(F_W, 0, 0, 0);
    o1 = o1 + K[23]*A(F_W, 0, 0, 0);
    o2 = o2 + K[35]*A(F_W, 0, 0, 0);
    out[0] = o0;
    out[1] = o1;
    out[2] = o2;
    out[3] = o3;
    out[4] = o4;
    out[5] = o5;
  }
  template <typename C, class Acc, class KT>
  __device__ __forceinline__ static void velocity(const Acc &A, const KT &K, C out[3]) {
    C o0 = K[0]*A(F_TXX, 1, 0, 0);
    C o1 = -K[12]*A(F_TXY, 1, 0, 0);
    C o2 = -K[24]*A(F_TXZ, 1, 0, 0);
    o0 = o0 - K[1]*A(F_TXX, 2, 0, 0);
    o1 = o1 - K[13]*A(F_TXY, -1, 0, 0);
    o2 = o2 - K[25]*A(F_TXZ, -1, 0, 0);
    o0 = o0 + K[2]*A(F_TXX, -1, 0, 0);
    o1 = o1 + K[14]*A(F_TXY, -2, 0, 0);
    o2 = o2 + K[26]*A(F_TXZ, -2, 0, 0);
    o0 = o0 - K[3]*A(F_TXX, 0, 0, 0);
    o1 = o1 + K[15]*A(F_TXY, 0, 0, 0);
    o2 = o2 + K[27]*A(F_TXZ, 0, 0, 0);
    o0 = o0 - K[4]*A(F_TXY, 0, 1, 0);
    o1 = o1 + K[16]*A(F_TYY, 0, 1, 0);
    o2 = o2 - K[28]*A(F_TYZ, 0, 1, 0);
    o0 = o0 - K[5]*A(F_TXY, 0, -1, 0);
    o1 = o1 - K[17]*A(F_TYY, 0, 2, 0);
    o2 = o2 - K[29]*A(F_TYZ, 0, -1, 0);
    o0 = o0 + K[6]*A(F_TXY, 0, -2, 0);
    o1 = o1 + K[18]*A(F_TYY, 0, -1, 0);
    o2 = o2 + K[30]*A(F_TYZ, 0, -2, 0);
    o0 = o0 + K[7]*A(F_TXY, 0, 0, 0);
    o1 = o1 - K[19]*A(F_TYY, 0, 0, 0);
    o2 = o2 + K[31]*A(F_TYZ, 0, 0, 0);
    o0 = o0 - K[8]*A(F_TXZ, 0, 0, 1);
    o1 = o1 - K[20]*A(F_TYZ, 0, 0, 1);
    o2 = o2 + K[32]*A(F_TZZ, 0, 0, 1);
    o0 = o0 - K[9]*A(F_TXZ, 0, 0, -1);
    o1 = o1 - K[21]*A(F_TYZ, 0, 0, -1);
    o2 = o2 - K[33]*A(F_TZZ, 0, 0, 2);
    o0 = o0 + K[10]*A(F_TXZ, 0, 0, -2);
    o1 = o1 + K[22]*A(F_TYZ, 0, 0, -2);
    o2 = o2 + K[34]*A(F_TZZ, 0, 0, -1);
    o0 = o0 + K[11]*A(F_TXZ, 0, 0, 0);
    o1 = o1 + K[23]*A(F_TYZ, 0, 0, 0);
    o2 = o2 - K[35]*A(F_TZZ, 0, 0, 0);
    o0 = o0 + A(F_U, 0, 0, 0);
    o1 = o1 + A(F_V, 0, 0, 0);
    o2 = o2 + A(F_W, 0, 0, 0);
    out[0] = o0;
    out[1] = o1;
    out[2] = o2;
  }
};

template <> struct GenSweep<2, 1> {
  static constexpr bool ok = true;
  static constexpr int NK_STRESS = 72, NK_VELOCITY = 36;
  template <typename C, class Acc, class KT>
  __device__ __forceinline__ static void stress(const Acc &A, const KT &K, C out[6]) {
    C o0 = A(F_TXX, 0, 0, 0);
    C o1 = A(F_TYY, 0, 0, 0);
    C o2 = A(F_TZZ, 0, 0, 0);
    C o3 = A(F_TXY, 0, 0, 0);
    C o4 = A(F_TYZ, 0, 0, 0);
    C o5 = A(F_TXZ, 0, 0, 0);
    o0 = o0 - K[0]*A(F_U, 1, 0, 0)*A.m(M_LAM);
    o1 = o1 - K[16]*A(F_U, 1, 0, 0)*A.m(M_LAM);
    o2 = o2 - K[32]*A(F_U, 1, 0, 0)*A.m(M_LAM);
    o3 = o3 + K[48]*A(F_U, 0, 1, 0)*A.m(M_MU12);
    o4 = o4 + K[56]*A(F_V, 0, 0, 1)*A.m(M_MU23);
    o5 = o5 + K[64]*A(F_U, 0, 0, 1)*A.m(M_MU13);
    o0 = o0 - K[1]*A(F_U, 1, 0, 0)*A.m(M_MU);
    o1 = o1 - K[17]*A(F_U, -1, 0, 0)*A.m(M_LAM);
    o2 = o2 - K[33]*A(F_U, -1, 0, 0)*A.m(M_LAM);
    o3 = o3 - K[49]*A(F_U, 0, 2, 0)*A.m(M_MU12);
    o4 = o4 - K[57]*A(F_V, 0, 0, 2)*A.m(M_MU23);
    o5 = o5 - K[65]*A(F_U, 0, 0, 2)*A.m(M_MU13);
    o0 = o0 - K[2]*A(F_U, -1, 0, 0)*A.m(M_LAM);
    o1 = o1 + K[18]*A(F_U, -2, 0, 0)*A.m(M_LAM);
    o2 = o2 + K[34]*A(F_U, -2, 0, 0)*A.m(M_LAM);
    o3 = o3 + K[50]*A(F_U, 0, -1, 0)*A.m(M_MU12);
    o4 = o4 + K[58]*A(F_V, 0, 0, -1)*A.m(M_MU23);
    o5 = o5 + K[66]*A(F_U, 0, 0, -1)*A.m(M_MU13);
    o0 = o0 - K[3]*A(F_U, -1, 0, 0)*A.m(M_MU);
    o1 = o1 + K[19]*A(F_U, 0, 0, 0)*A.m(M_LAM);
    o2 = o2 + K[35]*A(F_U, 0, 0, 0)*A.m(M_LAM);
    o3 = o3 - K[51]*A(F_U, 0, 0, 0)*A.m(M_MU12);
    o4 = o4 - K[59]*A(F_V, 0, 0, 0)*A.m(M_MU23);
    o5 = o5 - K[67]*A(F_U, 0, 0, 0)*A.m(M_MU13);
    o0 = o0 + K[4]*A(F_U, -2, 0, 0)*A.m(M_LAM);
    o1 = o1 - K[20]*A(F_V, 0, 1, 0)*A.m(M_LAM);
    o2 = o2 - K[36]*A(F_V, 0, 1, 0)*A.m(M_LAM);
    o3 = o3 + K[52]*A(F_V, 1, 0, 0)*A.m(M_MU12);
    o4 = o4 + K[60]*A(F_W, 0, 1, 0)*A.m(M_MU23);
    o5 = o5 + K[68]*A(F_W, 1, 0, 0)*A.m(M_MU13);
    o0 = o0 + K[5]*A(F_U, -2, 0, 0)*A.m(M_MU);
    o1 = o1 - K[21]*A(F_V, 0, 1, 0)*A.m(M_MU);
    o2 = o2 - K[37]*A(F_V, 0, -1, 0)*A.m(M_LAM);
    o3 = o3 - K[53]*A(F_V, 2, 0, 0)*A.m(M_MU12);
    o4 = o4 - K[61]*A(F_W, 0, 2, 0)*A.m(M_MU23);
    o5 = o5 - K[69]*A(F_W, 2, 0, 0)*A.m(M_MU13);
    o0 = o0 + K[6]*A(F_U, 0, 0, 0)*A.m(M_LAM);
    o1 = o1 - K[22]*A(F_V, 0, -1, 0)*A.m(M_LAM);
    o2 = o2 + K[38]*A(F_V, 0, -2, 0)*A.m(M_LAM);
    o3 = o3 + K[54]*A(F_V, -1, 0, 0)*A.m(M_MU12);
    o4 = o4 + K[62]*A(F_W, 0, -1, 0)*A.m(M_MU23);
    o5 = o5 + K[70]*A(F_W, -1, 0, 0)*A.m(M_MU13);
    o0 = o0 + K[7]*A(F_U, 0, 0, 0)*A.m(M_MU);
    o1 = o1 - K[23]*A(F_V, 0, -1, 0)*A.m(M_MU);
    o2 = o2 + K[39]*A(F_V, 0, 0, 0)*A.m(M_LAM);
    o3 = o3 - K[55]*A(F_V, 0, 0, 0)*A.m(M_MU12);
    o4 = o4 - K[63]*A(F_W, 0, 0, 0)*A.m(M_MU23);
    o5 = o5 - K[71]*A(F_W, 0, 0, 0)*A.m(M_MU13);
    o0 = o0 - K[8]*A(F_V, 0, 1, 0)*A.m(M_LAM);
    o1 = o1 + K[24]*A(F_V, 0, -2, 0)*A.m(M_LAM);
    o2 = o2 - K[40]*A(F_W, 0, 0, 1)*A.m(M_LAM);
    o0 = o0 - K[9]*A(F_V, 0, -1, 0)*A.m(M_LAM);
    o1 = o1 + K[25]*A(F_V, 0, -2, 0)*A.m(M_MU);
    o2 = o2 - K[41]*A(F_W, 0, 0, 1)*A.m(M_MU);
    o0 = o0 + K[10]*A(F_V, 0, -2, 0)*A.m(M_LAM);
    o1 = o1 + K[26]*A(F_V, 0, 0, 0)*A.m(M_LAM);
    o2 = o2 - K[42]*A(F_W, 0, 0, -1)*A.m(M_LAM);
    o0 = o0 + K[11]*A(F_V, 0, 0, 0)*A.m(M_LAM);
    o1 = o1 + K[27]*A(F_V, 0, 0, 0)*A.m(M_MU);
    o2 = o2 - K[43]*A(F_W, 0, 0, -1)*A.m(M_MU);
    o0 = o0 - K[12]*A(F_W, 0, 0, 1)*A.m(M_LAM);
    o1 = o1 - K[28]*A(F_W, 0, 0, 1)*A.m(M_LAM);
    o2 = o2 + K[44]*A(F_W, 0, 0, -2)*A.m(M_LAM);
    o0 = o0 - K[13]*A(F_W, 0, 0, -1)*A.m(M_LAM);
    o1 = o1 - K[29]*A(F_W, 0, 0, -1)*A.m(M_LAM);
    o2 = o2 + K[45]*A(F_W, 0, 0, -2)*A.m(M_MU);
    o0 = o0 + K[14]*A(F_W, 0, 0, -2)*A.m(M_LAM);
    o1 = o1 + K[30]*A(F_W, 0, 0, -2)*A.m(M_LAM);
    o2 = o2 + K[46]*A(F_W, 0, 0, 0)*A.m(M_LAM);
    o0 = o0 + K[15]*A(F_W, 0, 0, 0)*A.m(M_LAM);
    o1 = o1 + K[31]*A(F_W, 0, 0, 0)*A.m(M_LAM);
    o2 = o2 + K[47]*A(F_W, 0, 0, 0)*A.m(M_MU);
    out[0] = o0;
    out[1] = o1;
    out[2] = o2;
    out[3] = o3;
    out[4] = o4;
    out[5] = o5;
  }
  template <typename C, class Acc, class KT>
  __device__ __forceinline__ static void velocity(const Acc &A, const KT &K, C out[3]) {
    C o0 = K[0]*A(F_TXX, 1, 0, 0)*A.m(M_B1);
    C o1 = -K[12]*A(F_TXY, 1, 0, 0)*A.m(M_B2);
    C o2 = -K[24]*A(F_TXZ, 1, 0, 0)*A.m(M_B3);
    o0 = o0 - K[1]*A(F_TXX, 2, 0, 0)*A.m(M_B1);
    o1 = o1 - K[13]*A(F_TXY, -1, 0, 0)*A.m(M_B2);
    o2 = o2 - K[25]*A(F_TXZ, -1, 0, 0)*A.m(M_B3);
    o0 = o0 + K[2]*A(F_TXX, -1, 0, 0)*A.m(M_B1);
    o1 = o1 + K[14]*A(F_TXY, -2, 0, 0)*A.m(M_B2);
    o2 = o2 + K[26]*A(F_TXZ, -2, 0, 0)*A.m(M_B3);
    o0 = o0 - K[3]*A(F_TXX, 0, 0, 0)*A.m(M_B1);
    o1 = o1 + K[15]*A(F_TXY, 0, 0, 0)*A.m(M_B2);
    o2 = o2 + K[27]*A(F_TXZ, 0, 0, 0)*A.m(M_B3);
    o0 = o0 - K[4]*A(F_TXY, 0, 1, 0)*A.m(M_B1);
    o1 = o1 + K[16]*A(F_TYY, 0, 1, 0)*A.m(M_B2);
    o2 = o2 - K[28]*A(F_TYZ, 0, 1, 0)*A.m(M_B3);
    o0 = o0 - K[5]*A(F_TXY, 0, -1, 0)*A.m(M_B1);
    o1 = o1 - K[17]*A(F_TYY, 0, 2, 0)*A.m(M_B2);
    o2 = o2 - K[29]*A(F_TYZ, 0, -1, 0)*A.m(M_B3);
    o0 = o0 + K[6]*A(F_TXY, 0, -2, 0)*A.m(M_B1);
    o1 = o1 + K[18]*A(F_TYY, 0, -1, 0)*A.m(M_B2);
    o2 = o2 + K[30]*A(F_TYZ, 0, -2, 0)*A.m(M_B3);
    o0 = o0 + K[7]*A(F_TXY, 0, 0, 0)*A.m(M_B1);
    o1 = o1 - K[19]*A(F_TYY, 0, 0, 0)*A.m(M_B2);
    o2 = o2 + K[31]*A(F_TYZ, 0, 0, 0)*A.m(M_B3);
    o0 = o0 - K[8]*A(F_TXZ, 0, 0, 1)*A.m(M_B1);
    o1 = o1 - K[20]*A(F_TYZ, 0, 0, 1)*A.m(M_B2);
    o2 = o2 + K[32]*A(F_TZZ, 0, 0, 1)*A.m(M_B3);
    o0 = o0 - K[9]*A(F_TXZ, 0, 0, -1)*A.m(M_B1);
    o1 = o1 - K[21]*A(F_TYZ, 0, 0, -1)*A.m(M_B2);
    o2 = o2 - K[33]*A(F_TZZ, 0, 0, 2)*A.m(M_B3);
    o0 = o0 + K[10]*A(F_TXZ, 0, 0, -2)*A.m(M_B1);
    o1 = o1 + K[22]*A(F_TYZ, 0, 0, -2)*A.m(M_B2);
    o2 = o2 + K[34]*A(F_TZZ, 0, 0, -1)*A.m(M_B3);
    o0 = o0 + K[11]*A(F_TXZ, 0, 0, 0)*A.m(M_B1);
    o1 = o1 + K[23]*A(F_TYZ, 0, 0, 0)*A.m(M_B2);
    o2 = o2 - K[35]*A(F_TZZ, 0, 0, 0)*A.m(M_B3);
    o0 = o0 + A(F_U, 0, 0, 0);
    o1 = o1 + A(F_V, 0, 0, 0);
    o2 = o2 + A(F_W, 0, 0, 0);
    out[0] = o0;
    out[1] = o1;
    out[2] = o2;
  }
};

template <> struct GenSweep<3, 0> {
  static constexpr bool ok = true;
  static constexpr int NK_STRESS = 90, NK_VELOCITY = 54;
  template <typename C, class Acc, class KT>
  __device__ __forceinline__ static void stress(const Acc &A, const KT &K, C out[6]) {
    out[0] = A(F_TXX, 0, 0, 0) - K[0]*A(F_U, 1, 0, 0) + K[1]*A(F_U, 2, 0, 0) - K[2]*A(F_U, -1, 0, 0) + K[3]*A(F_U, -2, 0, 0) - K[4]*A(F_U, -3, 0, 0) + K[5]*A(F_U, 0, 0, 0) - K[6]*A(F_V, 0, 1, 0) + K[7]*A(F_V, 0, 2, 0) - K[8]*A(F_V, 0, -1, 0) + K[9]*A(F_V, 0, -2, 0) - K[10]*A(F_V, 0, -3, 0) + K[11]*A(F_V, 0, 0, 0) - K[12]*A(F_W, 0, 0, 1) + K[13]*A(F_W, 0, 0, 2) - K[14]*A(F_W, 0, 0, -1) + K[15]*A(F_W, 0, 0, -2) - K[16]*A(F_W, 0, 0, -3) + K[17]*A(F_W, 0, 0, 0);
    out[1] = A(F_TYY, 0, 0, 0) - K[18]*A(F_U, 1, 0, 0) + K[19]*A(F_U, 2, 0, 0) - K[20]*A(F_U, -1, 0, 0) + K[21]*A(F_U, -2, 0, 0) - K[22]*A(F_U, -3, 0, 0) + K[23]*A(F_U, 0, 0, 0) - K[24]*A(F_V, 0, 1, 0) + K[25]*A(F_V, 0, 2, 0) - K[26]*A(F_V, 0, -1, 0) + K[27]*A(F_V, 0, -2, 0) - K[28]*A(F_V, 0, -3, 0) + K[29]*A(F_V, 0, 0, 0) - K[30]*A(F_W, 0, 0, 1) + K[31]*A(F_W, 0, 0, 2) - K[32]*A(F_W, 0, 0, -1) + K[33]*A(F_W, 0, 0, -2) - K[34]*A(F_W, 0, 0, -3) + K[35]*A(F_W, 0, 0, 0);
    out[2] = A(F_TZZ, 0, 0, 0) - K[36]*A(F_U, 1, 0, 0) + K[37]*A(F_U, 2, 0, 0) - K[38]*A(F_U, -1, 0, 0) + K[39]*A(F_U, -2, 0, 0) - K[40]*A(F_U, -3, 0, 0) + K[41]*A(F_U, 0, 0, 0) - K[42]*A(F_V, 0, 1, 0) + K[43]*A(F_V, 0, 2, 0) - K[44]*A(F_V, 0, -1, 0) + K[45]*A(F_V, 0, -2, 0) - K[46]*A(F_V, 0, -3, 0) + K[47]*A(F_V, 0, 0, 0) - K[48]*A(F_W, 0, 0, 1) + K[49]*A(F_W, 0, 0, 2) - K[50]*A(F_W, 0, 0, -1) + K[51]*A(F_W, 0, 0, -2) - K[52]*A(F_W, 0, 0, -3) + K[53]*A(F_W, 0, 0, 0);
    out[3] = A(F_TXY, 0, 0, 0) + K[54]*A(F_U, 0, 1, 0) - K[55]*A(F_U, 0, 2, 0) + K[56]*A(F_U, 0, 3, 0) + K[57]*A(F_U, 0, -1, 0) - K[58]*A(F_U, 0, -2, 0) - K[59]*A(F_U, 0, 0, 0) + K[60]*A(F_V, 1, 0, 0) - K[61]*A(F_V, 2, 0, 0) + K[62]*A(F_V, 3, 0, 0) + K[63]*A(F_V, -1, 0, 0) - K[64]*A(F_V, -2, 0, 0) - K[65]*A(F_V, 0, 0, 0);
    out[4] = A(F_TYZ, 0, 0, 0) + K[66]*A(F_V, 0, 0, 1) - K[67]*A(F_V, 0, 0, 2) + K[68]*A(F_V, 0, 0, 3) + K[69]*A(F_V, 0, 0, -1) - K[70]*A(F_V, 0, 0, -2) - K[71]*A(F_V, 0, 0, 0) + K[72]*A(F_W, 0, 1, 0) - K[73]*A(F_W, 0, 2, 0) + K[74]*A(F_W, 0, 3, 0) + K[75]*A(F_W, 0, -1, 0) - K[76]*A(F_W, 0, -2, 0) - K[77]*A(F_W, 0, 0, 0);
    out[5] = A(F_TXZ, 0, 0, 0) + K[78]*A(F_U, 0, 0, 1) - K[79]*A(F_U, 0, 0, 2) + K[80]*A(F_U, 0, 0, 3) + K[81]*A(F_U, 0, 0, -1) - K[82]*A(F_U, 0, 0, -2) - K[83]*A(F_U, 0, 0, 0) + K[84]*A(F_W, 1, 0, 0) - K[85]*A(F_W, 2, 0, 0) + K[86]*A(F_W, 3, 0, 0) + K[87]*A(F_W, -1, 0, 0) - K[88]*A(F_W, -2, 0, 0) - K[89]*A(F_W, 0, 0, 0);
  }
  template <typename C, class Acc, class KT>
  __device__ __forceinline__ static void velocity(const Acc &A, const KT &K, C out[3]) {
    out[0] = K[0]*A(F_TXX, 1, 0, 0) - K[1]*A(F_TXX, 2, 0, 0) + K[2]*A(F_TXX, 3, 0, 0) + K[3]*A(F_TXX, -1, 0, 0) - K[4]*A(F_TXX, -2, 0, 0) - K[5]*A(F_TXX, 0, 0, 0) - K[6]*A(F_TXY, 0, 1, 0) + K[7]*A(F_TXY, 0, 2, 0) - K[8]*A(F_TXY, 0, -1, 0) + K[9]*A(F_TXY, 0, -2, 0) - K[10]*A(F_TXY, 0, -3, 0) + K[11]*A(F_TXY, 0, 0, 0) - K[12]*A(F_TXZ, 0, 0, 1) + K[13]*A(F_TXZ, 0, 0, 2) - K[14]*A(F_TXZ, 0, 0, -1) + K[15]*A(F_TXZ, 0, 0, -2) - K[16]*A(F_TXZ, 0, 0, -3) + K[17]*A(F_TXZ, 0, 0, 0) + A(F_U, 0, 0, 0);
    out[1] = -K[18]*A(F_TXY, 1, 0, 0) + K[19]*A(F_TXY, 2, 0, 0) - K[20]*A(F_TXY, -1, 0, 0) + K[21]*A(F_TXY, -2, 0, 0) - K[22]*A(F_TXY, -3, 0, 0) + K[23]*A(F_TXY, 0, 0, 0) + K[24]*A(F_TYY, 0, 1, 0) - K[25]*A(F_TYY, 0, 2, 0) + K[26]*A(F_TYY, 0, 3, 0) + K[27]*A(F_TYY, 0, -1, 0) - K[28]*A(F_TYY, 0, -2, 0) - K[29]*A(F_TYY, 0, 0, 0) - K[30]*A(F_TYZ, 0, 0, 1) + K[31]*A(F_TYZ, 0, 0, 2) - K[32]*A(F_TYZ, 0, 0, -1) + K[33]*A(F_TYZ, 0, 0, -2) - K[34]*A(F_TYZ, 0, 0, -3) + K[35]*A(F_TYZ, 0, 0, 0) + A(F_V, 0, 0, 0);
    out[2] = -K[36]*A(F_TXZ, 1, 0, 0) + K[37]*A(F_TXZ, 2, 0, 0) - K[38]*A(F_TXZ, -1, 0, 0) + K[39]*A(F_TXZ, -2, 0, 0) - K[40]*A(F_TXZ, -3, 0, 0) + K[41]*A(F_TXZ, 0, 0, 0) - K[42]*A(F_TYZ, 0, 1, 0) + K[43]*A(F_TYZ, 0, 2, 0) - K[44]*A(F_TYZ, 0, -1, 0) + K[45]*A(F_TYZ, 0, -2, 0) - K[46]*A(F_TYZ, 0, -3, 0) + K[47]*A(F_TYZ, 0, 0, 0) + K[48]*A(F_TZZ, 0, 0, 1) - K[49]*A(F_TZZ, 0, 0, 2) + K[50]*A(F_TZZ, 0, 0, 3) + K[51]*A(F_TZZ, 0, 0, -1) - K[52]*A(F_TZZ, 0, 0, -2) - K[53]*A(F_TZZ, 0, 0, 0) + A(F_W, 0, 0, 0);
  }
};

template <> struct GenSweep<3, 1> {
  static constexpr bool ok = true;
  static constexpr int NK_STRESS = 108, NK_VELOCITY = 54;
  template <typename C, class Acc, class KT>
  __device__ __forceinline__ static void stress(const Acc &A, const KT &K, C out[6]) {
    out[0] = A(F_TXX, 0, 0, 0) - K[0]*A(F_U, 1, 0, 0)*A.m(M_LAM) - K[1]*A(F_U, 1, 0, 0)*A.m(M_MU) + K[2]*A(F_U, 2, 0, 0)*A.m(M_LAM) + K[3]*A(F_U, 2, 0, 0)*A.m(M_MU) - K[4]*A(F_U, -1, 0, 0)*A.m(M_LAM) - K[5]*A(F_U, -1, 0, 0)*A.m(M_MU) + K[6]*A(F_U, -2, 0, 0)*A.m(M_LAM) + K[7]*A(F_U, -2, 0, 0)*A.m(M_MU) - K[8]*A(F_U, -3, 0, 0)*A.m(M_LAM) - K[9]*A(F_U, -3, 0, 0)*A.m(M_MU) + K[10]*A(F_U, 0, 0, 0)*A.m(M_LAM) + K[11]*A(F_U, 0, 0, 0)*A.m(M_MU) - K[12]*A(F_V, 0, 1, 0)*A.m(M_LAM) + K[13]*A(F_V, 0, 2, 0)*A.m(M_LAM) - K[14]*A(F_V, 0, -1, 0)*A.m(M_LAM) + K[15]*A(F_V, 0, -2, 0)*A.m(M_LAM) - K[16]*A(F_V, 0, -3, 0)*A.m(M_LAM) + K[17]*A(F_V, 0, 0, 0)*A.m(M_LAM) - K[18]*A(F_W, 0, 0, 1)*A.m(M_LAM) + K[19]*A(F_W, 0, 0, 2)*A.m(M_LAM) - K[20]*A(F_W, 0, 0, -1)*A.m(M_LAM) + K[21]*A(F_W, 0, 0, -2)*A.m(M_LAM) - K[22]*A(F_W, 0, 0, -3)*A.m(M_LAM) + K[23]*A(F_W, 0, 0, 0)*A.m(M_LAM);
    out[1] = A(F_TYY, 0, 0, 0) - K[24]*A(F_U, 1, 0, 0)*A.m(M_LAM) + K[25]*A(F_U, 2, 0, 0)*A.m(M_LAM) - K[26]*A(F_U, -1, 0, 0)*A.m(M_LAM) + K[27]*A(F_U, -2, 0, 0)*A.m(M_LAM) - K[28]*A(F_U, -3, 0, 0)*A.m(M_LAM) + K[29]*A(F_U, 0, 0, 0)*A.m(M_LAM) - K[30]*A(F_V, 0, 1, 0)*A.m(M_LAM) - K[31]*A(F_V, 0, 1, 0)*A.m(M_MU) + K[32]*A(F_V, 0, 2, 0)*A.m(M_LAM) + K[33]*A(F_V, 0, 2, 0)*A.m(M_MU) - K[34]*A(F_V, 0, -1, 0)*A.m(M_LAM) - K[35]*A(F_V, 0, -1, 0)*A.m(M_MU) + K[36]*A(F_V, 0, -2, 0)*A.m(M_LAM) + K[37]*A(F_V, 0, -2, 0)*A.m(M_MU) - K[38]*A(F_V, 0, -3, 0)*A.m(M_LAM) - K[39]*A(F_V, 0, -3, 0)*A.m(M_MU) + K[40]*A(F_V, 0, 0, 0)*A.m(M_LAM) + K[41]*A(F_V, 0, 0, 0)*A.m(M_MU) - K[42]*A(F_W, 0, 0, 1)*A.m(M_LAM) + K[43]*A(F_W, 0, 0, 2)*A.m(M_LAM) - K[44]*A(F_W, 0, 0, -1)*A.m(M_LAM) + K[45]*A(F_W, 0, 0, -2)*A.m(M_LAM) - K[46]*A(F_W, 0, 0, -3)*A.m(M_LAM) + K[47]*A(F_W, 0, 0, 0)*A.m(M_LAM);
    out[2] = A(F_TZZ, 0, 0, 0) - K[48]*A(F_U, 1, 0, 0)*A.m(M_LAM) + K[49]*A(F_U, 2, 0, 0)*A.m(M_LAM) - K[50]*A(F_U, -1, 0, 0)*A.m(M_LAM) + K[51]*A(F_U, -2, 0, 0)*A.m(M_LAM) - K[52]*A(F_U, -3, 0, 0)*A.m(M_LAM) + K[53]*A(F_U, 0, 0, 0)*A.m(M_LAM) - K[54]*A(F_V, 0, 1, 0)*A.m(M_LAM) + K[55]*A(F_V, 0, 2, 0)*A.m(M_LAM) - K[56]*A(F_V, 0, -1, 0)*A.m(M_LAM) + K[57]*A(F_V, 0, -2, 0)*A.m(M_LAM) - K[58]*A(F_V, 0, -3, 0)*A.m(M_LAM) + K[59]*A(F_V, 0, 0, 0)*A.m(M_LAM) - K[60]*A(F_W, 0, 0, 1)*A.m(M_LAM) - K[61]*A(F_W, 0, 0, 1)*A.m(M_MU) + K[62]*A(F_W, 0, 0, 2)*A.m(M_LAM) + K[63]*A(F_W, 0, 0, 2)*A.m(M_MU) - K[64]*A(F_W, 0, 0, -1)*A.m(M_LAM) - K[65]*A(F_W, 0, 0, -1)*A.m(M_MU) + K[66]*A(F_W, 0, 0, -2)*A.m(M_LAM) + K[67]*A(F_W, 0, 0, -2)*A.m(M_MU) - K[68]*A(F_W, 0, 0, -3)*A.m(M_LAM) - K[69]*A(F_W, 0, 0, -3)*A.m(M_MU) + K[70]*A(F_W, 0, 0, 0)*A.m(M_LAM) + K[71]*A(F_W, 0, 0, 0)*A.m(M_MU);
    out[3] = A(F_TXY, 0, 0, 0) + K[72]*A(F_U, 0, 1, 0)*A.m(M_MU12) - K[73]*A(F_U, 0, 2, 0)*A.m(M_MU12) + K[74]*A(F_U, 0, 3, 0)*A.m(M_MU12) + K[75]*A(F_U, 0, -1, 0)*A.m(M_MU12) - K[76]*A(F_U, 0, -2, 0)*A.m(M_MU12) - K[77]*A(F_U, 0, 0, 0)*A.m(M_MU12) + K[78]*A(F_V, 1, 0, 0)*A.m(M_MU12) - K[79]*A(F_V, 2, 0, 0)*A.m(M_MU12) + K[80]*A(F_V, 3, 0, 0)*A.m(M_MU12) + K[81]*A(F_V, -1, 0, 0)*A.m(M_MU12) - K[82]*A(F_V, -2, 0, 0)*A.m(M_MU12) - K[83]*A(F_V, 0, 0, 0)*A.m(M_MU12);
    out[4] = A(F_TYZ, 0, 0, 0) + K[84]*A(F_V, 0, 0, 1)*A.m(M_MU23) - K[85]*A(F_V, 0, 0, 2)*A.m(M_MU23) + K[86]*A(F_V, 0, 0, 3)*A.m(M_MU23) + K[87]*A(F_V, 0, 0, -1)*A.m(M_MU23) - K[88]*A(F_V, 0, 0, -2)*A.m(M_MU23) - K[89]*A(F_V, 0, 0, 0)*A.m(M_MU23) + K[90]*A(F_W, 0, 1, 0)*A.m(M_MU23) - K[91]*A(F_W, 0, 2, 0)*A.m(M_MU23) + K[92]*A(F_W, 0, 3, 0)*A.m(M_MU23) + K[93]*A(F_W, 0, -1, 0)*A.m(M_MU23) - K[94]*A(F_W, 0, -2, 0)*A.m(M_MU23) - K[95]*A(F_W, 0, 0, 0)*A.m(M_MU23);
    out[5] = A(F_TXZ, 0, 0, 0) + K[96]*A(F_U, 0, 0, 1)*A.m(M_MU13) - K[97]*A(F_U, 0, 0, 2)*A.m(M_MU13) + K[98]*A(F_U, 0, 0, 3)*A.m(M_MU13) + K[99]*A(F_U, 0, 0, -1)*A.m(M_MU13) - K[100]*A(F_U, 0, 0, -2)*A.m(M_MU13) - K[101]*A(F_U, 0, 0, 0)*A.m(M_MU13) + K[102]*A(F_W, 1, 0, 0)*A.m(M_MU13) - K[103]*A(F_W, 2, 0, 0)*A.m(M_MU13) + K[104]*A(F_W, 3, 0, 0)*A.m(M_MU13) + K[105]*A(F_W, -1, 0, 0)*A.m(M_MU13) - K[106]*A(F_W, -2, 0, 0)*A.m(M_MU13) - K[107]*A(F_W, 0, 0, 0)*A.m(M_MU13);
  }
  template <typename C, class Acc, class KT>
  __device__ __forceinline__ static void velocity(const Acc &A, const KT &K, C out[3]) {
    out[0] = K[0]*A(F_TXX, 1, 0, 0)*A.m(M_B1) - K[1]*A(F_TXX, 2, 0, 0)*A.m(M_B1) + K[2]*A(F_TXX, 3, 0, 0)*A.m(M_B1) + K[3]*A(F_TXX, -1, 0, 0)*A.m(M_B1) - K[4]*A(F_TXX, -2, 0, 0)*A.m(M_B1) - K[5]*A(F_TXX, 0, 0, 0)*A.m(M_B1) - K[6]*A(F_TXY, 0, 1, 0)*A.m(M_B1) + K[7]*A(F_TXY, 0, 2, 0)*A.m(M_B1) - K[8]*A(F_TXY, 0, -1, 0)*A.m(M_B1) + K[9]*A(F_TXY, 0, -2, 0)*A.m(M_B1) - K[10]*A(F_TXY, 0, -3, 0)*A.m(M_B1) + K[11]*A(F_TXY, 0, 0, 0)*A.m(M_B1) - K[12]*A(F_TXZ, 0, 0, 1)*A.m(M_B1) + K[13]*A(F_TXZ, 0, 0, 2)*A.m(M_B1) - K[14]*A(F_TXZ, 0, 0, -1)*A.m(M_B1) + K[15]*A(F_TXZ, 0, 0, -2)*A.m(M_B1) - K[16]*A(F_TXZ, 0, 0, -3)*A.m(M_B1) + K[17]*A(F_TXZ, 0, 0, 0)*A.m(M_B1) + A(F_U, 0, 0, 0);
    out[1] = -K[18]*A(F_TXY, 1, 0, 0)*A.m(M_B2) + K[19]*A(F_TXY, 2, 0, 0)*A.m(M_B2) - K[20]*A(F_TXY, -1, 0, 0)*A.m(M_B2) + K[21]*A(F_TXY, -2, 0, 0)*A.m(M_B2) - K[22]*A(F_TXY, -3, 0, 0)*A.m(M_B2) + K[23]*A(F_TXY, 0, 0, 0)*A.m(M_B2) + K[24]*A(F_TYY, 0, 1, 0)*A.m(M_B2) - K[25]*A(F_TYY, 0, 2, 0)*A.m(M_B2) + K[26]*A(F_TYY, 0, 3, 0)*A.m(M_B2) + K[27]*A(F_TYY, 0, -1, 0)*A.m(M_B2) - K[28]*A(F_TYY, 0, -2, 0)*A.m(M_B2) - K[29]*A(F_TYY, 0, 0, 0)*A.m(M_B2) - K[30]*A(F_TYZ, 0, 0, 1)*A.m(M_B2) + K[31]*A(F_TYZ, 0, 0, 2)*A.m(M_B2) - K[32]*A(F_TYZ, 0, 0, -1)*A.m(M_B2) + K[33]*A(F_TYZ, 0, 0, -2)*A.m(M_B2) - K[34]*A(F_TYZ, 0, 0, -3)*A.m(M_B2) + K[35]*A(F_TYZ, 0, 0, 0)*A.m(M_B2) + A(F_V, 0, 0, 0);
    out[2] = -K[36]*A(F_TXZ, 1, 0, 0)*A.m(M_B3) + K[37]*A(F_TXZ, 2, 0, 0)*A.m(M_B3) - K[38]*A(F_TXZ, -1, 0, 0)*A.m(M_B3) + K[39]*A(F_TXZ, -2, 0, 0)*A.m(M_B3) - K[40]*A(F_TXZ, -3, 0, 0)*A.m(M_B3) + K[41]*A(F_TXZ, 0, 0, 0)*A.m(M_B3) - K[42]*A(F_TYZ, 0, 1, 0)*A.m(M_B3) + K[43]*A(F_TYZ, 0, 2, 0)*A.m(M_B3) - K[44]*A(F_TYZ, 0, -1, 0)*A.m(M_B3) + K[45]*A(F_TYZ, 0, -2, 0)*A.m(M_B3) - K[46]*A(F_TYZ, 0, -3, 0)*A.m(M_B3) + K[47]*A(F_TYZ, 0, 0, 0)*A.m(M_B3) + K[48]*A(F_TZZ, 0, 0, 1)*A.m(M_B3) - K[49]*A(F_TZZ, 0, 0, 2)*A.m(M_B3) + K[50]*A(F_TZZ, 0, 0, 3)*A.m(M_B3) + K[51]*A(F_TZZ, 0, 0, -1)*A.m(M_B3) - K[52]*A(F_TZZ, 0, 0, -2)*A.m(M_B3) - K[53]*A(F_TZZ, 0, 0, 0)*A.m(M_B3) + A(F_W, 0, 0, 0);
  }
};

template <> struct GenSweep<4, 0> {
  static constexpr bool ok = true;
  static constexpr int NK_STRESS = 120, NK_VELOCITY = 72;
  template <typename C, class Acc, class KT>
  __device__ __forceinline__ static void stress(const Acc &A, const KT &K, C out[6]) {
    out[0] = A(F_TXX, 0, 0, 0) - K[0]*A(F_U, 1, 0, 0) + K[1]*A(F_U, 2, 0, 0) - K[2]*A(F_U, 3, 0, 0) - K[3]*A(F_U, -1, 0, 0) + K[4]*A(F_U, -2, 0, 0) - K[5]*A(F_U, -3, 0, 0) + K[6]*A(F_U, -4, 0, 0) + K[7]*A(F_U, 0, 0, 0) - K[8]*A(F_V, 0, 1, 0) + K[9]*A(F_V, 0, 2, 0) - K[10]*A(F_V, 0, 3, 0) - K[11]*A(F_V, 0, -1, 0) + K[12]*A(F_V, 0, -2, 0) - K[13]*A(F_V, 0, -3, 0) + K[14]*A(F_V, 0, -4, 0) + K[15]*A(F_V, 0, 0, 0) - K[16]*A(F_W, 0, 0, 1) + K[17]*A(F_W, 0, 0, 2) - K[18]*A(F_W, 0, 0, 3) - K[19]*A(F_W, 0, 0, -1) + K[20]*A(F_W, 0, 0, -2) - K[21]*A(F_W, 0, 0, -3) + K[22]*A(F_W, 0, 0, -4) + K[23]*A(F_W, 0, 0, 0);
    out[1] = A(F_TYY, 0, 0, 0) - K[24]*A(F_U, 1, 0, 0) + K[25]*A(F_U, 2, 0, 0) - K[26]*A(F_U, 3, 0, 0) - K[27]*A(F_U, -1, 0, 0) + K[28]*A(F_U, -2, 0, 0) - K[29]*A(F_U, -3, 0, 0) + K[30]*A(F_U, -4, 0, 0) + K[31]*A(F_U, 0, 0, 0) - K[32]*A(F_V, 0, 1, 0) + K[33]*A(F_V, 0, 2, 0) - K[34]*A(F_V, 0, 3, 0) - K[35]*A(F_V, 0, -1, 0) + K[36]*A(F_V, 0, -2, 0) - K[37]*A(F_V, 0, -3, 0) + K[38]*A(F_V, 0, -4, 0) + K[39]*A(F_V, 0, 0, 0) - K[40]*A(F_W, 0, 0, 1) + K[41]*A(F_W, 0, 0, 2) - K[42]*A(F_W, 0, 0, 3) - K[43]*A(F_W, 0, 0, -1) + K[44]*A(F_W, 0, 0, -2) - K[45]*A(F_W, 0, 0, -3) + K[46]*A(F_W, 0, 0, -4) + K[47]*A(F_W, 0, 0, 0);
    out[2] = A(F_TZZ, 0, 0, 0) - K[48]*A(F_U, 1, 0, 0) + K[49]*A(F_U, 2, 0, 0) - K[50]*A(F_U, 3, 0, 0) - K[51]*A(F_U, -1, 0, 0) + K[52]*A(F_U, -2, 0, 0) - K[53]*A(F_U, -3, 0, 0) + K[54]*A(F_U, -4, 0, 0) + K[55]*A(F_U, 0, 0, 0) - K[56]*A(F_V, 0, 1, 0) + K[57]*A(F_V, 0, 2, 0) - K[58]*A(F_V, 0, 3, 0) - K[59]*A(F_V, 0, -1, 0) + K[60]*A(F_V, 0, -2, 0) - K[61]*A(F_V, 0, -3, 0) + K[62]*A(F_V, 0, -4, 0) + K[63]*A(F_V, 0, 0, 0) - K[64]*A(F_W, 0, 0, 1) + K[65]*A(F_W, 0, 0, 2) - K[66]*A(F_W, 0, 0, 3) - K[67]*A(F_W, 0, 0, -1) + K[68]*A(F_W, 0, 0, -2) - K[69]*A(F_W, 0, 0, -3) + K[70]*A(F_W, 0, 0, -4) + K[71]*A(F_W, 0, 0, 0);
    out[3] = A(F_TXY, 0, 0, 0) + K[72]*A(F_U, 0, 1, 0) - K[73]*A(F_U, 0, 2, 0) + K[74]*A(F_U, 0, 3, 0) - K[75]*A(F_U, 0, 4, 0) + K[76]*A(F_U, 0, -1, 0) - K[77]*A(F_U, 0, -2, 0) + K[78]*A(F_U, 0, -3, 0) - K[79]*A(F_U, 0, 0, 0) + K[80]*A(F_V, 1, 0, 0) - K[81]*A(F_V, 2, 0, 0) + K[82]*A(F_V, 3, 0, 0) - K[83]*A(F_V, 4, 0, 0) + K[84]*A(F_V, -1, 0, 0) - K[85]*A(F_V, -2, 0, 0) + K[86]*A(F_V, -3, 0, 0) - K[87]*A(F_V, 0, 0, 0);
    out[4] = A(F_TYZ, 0, 0, 0) + K[88]*A(F_V, 0, 0, 1) - K[89]*A(F_V, 0, 0, 2) + K[90]*A(F_V, 0, 0, 3) - K[91]*A(F_V, 0, 0, 4) + K[92]*A(F_V, 0, 0, -1) - K[93]*A(F_V, 0, 0, -2) + K[94]*A(F_V, 0, 0, -3) - K[95]*A(F_V, 0, 0, 0) + K[96]*A(F_W, 0, 1, 0) - K[97]*A(F_W, 0, 2, 0) + K[98]*A(F_W, 0, 3, 0) - K[99]*A(F_W, 0, 4, 0) + K[100]*A(F_W, 0, -1, 0) - K[101]*A(F_W, 0, -2, 0) + K[102]*A(F_W, 0, -3, 0) - K[103]*A(F_W, 0, 0, 0);
    out[5] = A(F_TXZ, 0, 0, 0) + K[104]*A(F_U, 0, 0, 1) - K[105]*A(F_U, 0, 0, 2) + K[106]*A(F_U, 0, 0, 3) - K[107]*A(F_U, 0, 0, 4) + K[108]*A(F_U, 0, 0, -1) - K[109]*A(F_U, 0, 0, -2) + K[110]*A(F_U, 0, 0, -3) - K[111]*A(F_U, 0, 0, 0) + K[112]*A(F_W, 1, 0, 0) - K[113]*A(F_W, 2, 0, 0) + K[114]*A(F_W, 3, 0, 0) - K[115]*A(F_W, 4, 0, 0) + K[116]*A(F_W, -1, 0, 0) - K[117]*A(F_W, -2, 0, 0) + K[118]*A(F_W, -3, 0, 0) - K[119]*A(F_W, 0, 0, 0);
  }
  template <typename C, class Acc, class KT>
  __device__ __forceinline__ static void velocity(const Acc &A, const KT &K, C out[3]) {
    out[0] = K[0]*A(F_TXX, 1, 0, 0) - K[1]*A(F_TXX, 2, 0, 0) + K[2]*A(F_TXX, 3, 0, 0) - K[3]*A(F_TXX, 4, 0, 0) + K[4]*A(F_TXX, -1, 0, 0) - K[5]*A(F_TXX, -2, 0, 0) + K[6]*A(F_TXX, -3, 0, 0) - K[7]*A(F_TXX, 0, 0, 0) - K[8]*A(F_TXY, 0, 1, 0) + K[9]*A(F_TXY, 0, 2, 0) - K[10]*A(F_TXY, 0, 3, 0) - K[11]*A(F_TXY, 0, -1, 0) + K[12]*A(F_TXY, 0, -2, 0) - K[13]*A(F_TXY, 0, -3, 0) + K[14]*A(F_TXY, 0, -4, 0) + K[15]*A(F_TXY, 0, 0, 0) - K[16]*A(F_TXZ, 0, 0, 1) + K[17]*A(F_TXZ, 0, 0, 2) - K[18]*A(F_TXZ, 0, 0, 3) - K[19]*A(F_TXZ, 0, 0, -1) + K[20]*A(F_TXZ, 0, 0, -2) - K[21]*A(F_TXZ, 0, 0, -3) + K[22]*A(F_TXZ, 0, 0, -4) + K[23]*A(F_TXZ, 0, 0, 0) + A(F_U, 0, 0, 0);
    out[1] = -K[24]*A(F_TXY, 1, 0, 0) + K[25]*A(F_TXY, 2, 0, 0) - K[26]*A(F_TXY, 3, 0, 0) - K[27]*A(F_TXY, -1, 0, 0) + K[28]*A(F_TXY, -2, 0, 0) - K[29]*A(F_TXY, -3, 0, 0) + K[30]*A(F_TXY, -4, 0, 0) + K[31]*A(F_TXY, 0, 0, 0) + K[32]*A(F_TYY, 0, 1, 0) - K[33]*A(F_TYY, 0, 2, 0) + K[34]*A(F_TYY, 0, 3, 0) - K[35]*A(F_TYY, 0, 4, 0) + K[36]*A(F_TYY, 0, -1, 0) - K[37]*A(F_TYY, 0, -2, 0) + K[38]*A(F_TYY, 0, -3, 0) - K[39]*A(F_TYY, 0, 0, 0) - K[40]*A(F_TYZ, 0, 0, 1) + K[41]*A(F_TYZ, 0, 0, 2) - K[42]*A(F_TYZ, 0, 0, 3) - K[43]*A(F_TYZ, 0, 0, -1) + K[44]*A(F_TYZ, 0, 0, -2) - K[45]*A(F_TYZ, 0, 0, -3) + K[46]*A(F_TYZ, 0, 0, -4) + K[47]*A(F_TYZ, 0, 0, 0) + A(F_V, 0, 0, 0);
    out[2] = -K[48]*A(F_TXZ, 1, 0, 0) + K[49]*A(F_TXZ, 2, 0, 0) - K[50]*A(F_TXZ, 3, 0, 0) - K[51]*A(F_TXZ, -1, 0, 0) + K[52]*A(F_TXZ, -2, 0, 0) - K[53]*A(F_TXZ, -3, 0, 0) + K[54]*A(F_TXZ, -4, 0, 0) + K[55]*A(F_TXZ, 0, 0, 0) - K[56]*A(F_TYZ, 0, 1, 0) + K[57]*A(F_TYZ, 0, 2, 0) - K[58]*A(F_TYZ, 0, 3, 0) - K[59]*A(F_TYZ, 0, -1, 0) + K[60]*A(F_TYZ, 0, -2, 0) - K[61]*A(F_TYZ, 0, -3, 0) + K[62]*A(F_TYZ, 0, -4, 0) + K[63]*A(F_TYZ, 0, 0, 0) + K[64]*A(F_TZZ, 0, 0, 1) - K[65]*A(F_TZZ, 0, 0, 2) + K[66]*A(F_TZZ, 0, 0, 3) - K[67]*A(F_TZZ, 0, 0, 4) + K[68]*A(F_TZZ, 0, 0, -1) - K[69]*A(F_TZZ, 0, 0, -2) + K[70]*A(F_TZZ, 0, 0, -3) - K[71]*A(F_TZZ, 0, 0, 0) + A(F_W, 0, 0, 0);
  }
};

template <> struct GenSweep<4, 1> {
  static constexpr bool ok = true;
  static constexpr int NK_STRESS = 144, NK_VELOCITY = 72;
  template <typename C, class Acc, class KT>
  __device__ __forceinline__ static void stress(const Acc &A, const KT &K, C out[6]) {
    out[0] = A(F_TXX, 0, 0, 0) - K[0]*A(F_U, 1, 0, 0)*A.m(M_LAM) - K[1]*A(F_U, 1, 0, 0)*A.m(M_MU) + K[2]*A(F_U, 2, 0, 0)*A.m(M_LAM) + K[3]*A(F_U, 2, 0, 0)*A.m(M_MU) - K[4]*A(F_U, 3, 0, 0)*A.m(M_LAM) - K[5]*A(F_U, 3, 0, 0)*A.m(M_MU) - K[6]*A(F_U, -1, 0, 0)*A.m(M_LAM) - K[7]*A(F_U, -1, 0, 0)*A.m(M_MU) + K[8]*A(F_U, -2, 0, 0)*A.m(M_LAM) + K[9]*A(F_U, -2, 0, 0)*A.m(M_MU) - K[10]*A(F_U, -3, 0, 0)*A.m(M_LAM) - K[11]*A(F_U, -3, 0, 0)*A.m(M_MU) + K[12]*A(F_U, -4, 0, 0)*A.m(M_LAM) + K[13]*A(F_U, -4, 0, 0)*A.m(M_MU) + K[14]*A(F_U, 0, 0, 0)*A.m(M_LAM) + K[15]*A(F_U, 0, 0, 0)*A.m(M_MU) - K[16]*A(F_V, 0, 1, 0)*A.m(M_LAM) + K[17]*A(F_V, 0, 2, 0)*A.m(M_LAM) - K[18]*A(F_V, 0, 3, 0)*A.m(M_LAM) - K[19]*A(F_V, 0, -1, 0)*A.m(M_LAM) + K[20]*A(F_V, 0, -2, 0)*A.m(M_LAM) - K[21]*A(F_V, 0, -3, 0)*A.m(M_LAM) + K[22]*A(F_V, 0, -4, 0)*A.m(M_LAM) + K[23]*A(F_V, 0, 0, 0)*A.m(M_LAM) - K[24]*A(F_W, 0, 0, 1)*A.m(M_LAM) + K[25]*A(F_W, 0, 0, 2)*A.m(M_LAM) - K[26]*A(F_W, 0, 0, 3)*A.m(M_LAM) - K[27]*A(F_W, 0, 0, -1)*A.m(M_LAM) + K[28]*A(F_W, 0, 0, -2)*A.m(M_LAM) - K[29]*A(F_W, 0, 0, -3)*A.m(M_LAM) + K[30]*A(F_W, 0, 0, -4)*A.m(M_LAM) + K[31]*A(F_W, 0, 0, 0)*A.m(M_LAM);
    out[1] = A(F_TYY, 0, 0, 0) - K[32]*A(F_U, 1, 0, 0)*A.m(M_LAM) + K[33]*A(F_U, 2, 0, 0)*A.m(M_LAM) - K[34]*A(F_U, 3, 0, 0)*A.m(M_LAM) - K[35]*A(F_U, -1, 0, 0)*A.m(M_LAM) + K[36]*A(F_U, -2, 0, 0)*A.m(M_LAM) - K[37]*A(F_U, -3, 0, 0)*A.m(M_LAM) + K[38]*A(F_U, -4, 0, 0)*A.m(M_LAM) + K[39]*A(F_U, 0, 0, 0)*A.m(M_LAM) - K[40]*A(F_V, 0, 1, 0)*A.m(M_LAM) - K[41]*A(F_V, 0, 1, 0)*A.m(M_MU) + K[42]*A(F_V, 0, 2, 0)*A.m(M_LAM) + K[43]*A(F_V, 0, 2, 0)*A.m(M_MU) - K[44]*A(F_V, 0, 3, 0)*A.m(M_LAM) - K[45]*A(F_V, 0, 3, 0)*A.m(M_MU) - K[46]*A(F_V, 0, -1, 0)*A.m(M_LAM) - K[47]*A(F_V, 0, -1, 0)*A.m(M_MU) + K[48]*A(F_V, 0, -2, 0)*A.m(M_LAM) + K[49]*A(F_V, 0, -2, 0)*A.m(M_MU) - K[50]*A(F_V, 0, -3, 0)*A.m(M_LAM) - K[51]*A(F_V, 0, -3, 0)*A.m(M_MU) + K[52]*A(F_V, 0, -4, 0)*A.m(M_LAM) + K[53]*A(F_V, 0, -4, 0)*A.m(M_MU) + K[54]*A(F_V, 0, 0, 0)*A.m(M_LAM) + K[55]*A(F_V, 0, 0, 0)*A.m(M_MU) - K[56]*A(F_W, 0, 0, 1)*A.m(M_LAM) + K[57]*A(F_W, 0, 0, 2)*A.m(M_LAM) - K[58]*A(F_W, 0, 0, 3)*A.m(M_LAM) - K[59]*A(F_W, 0, 0, -1)*A.m(M_LAM) + K[60]*A(F_W, 0, 0, -2)*A.m(M_LAM) - K[61]*A(F_W, 0, 0, -3)*A.m(M_LAM) + K[62]*A(F_W, 0, 0, -4)*A.m(M_LAM) + K[63]*A(F_W, 0, 0, 0)*A.m(M_LAM);
    out[2] = A(F_TZZ, 0, 0, 0) - K[64]*A(F_U, 1, 0, 0)*A.m(M_LAM) + K[65]*A(F_U, 2, 0, 0)*A.m(M_LAM) - K[66]*A(F_U, 3, 0, 0)*A.m(M_LAM) - K[67]*A(F_U, -1, 0, 0)*A.m(M_LAM) + K[68]*A(F_U, -2, 0, 0)*A.m(M_LAM) - K[69]*A(F_U, -3, 0, 0)*A.m(M_LAM) + K[70]*A(F_U, -4, 0, 0)*A.m(M_LAM) + K[71]*A(F_U, 0, 0, 0)*A.m(M_LAM) - K[72]*A(F_V, 0, 1, 0)*A.m(M_LAM) + K[73]*A(F_V, 0, 2, 0)*A.m(M_LAM) - K[74]*A(F_V, 0, 3, 0)*A.m(M_LAM) - K[75]*A(F_V, 0, -1, 0)*A.m(M_LAM) + K[76]*A(F_V, 0, -2, 0)*A.m(M_LAM) - K[77]*A(F_V, 0, -3, 0)*A.m(M_LAM) + K[78]*A(F_V, 0, -4, 0)*A.m(M_LAM) + K[79]*A(F_V, 0, 0, 0)*A.m(M_LAM) - K[80]*A(F_W, 0, 0, 1)*A.m(M_LAM) - K[81]*A(F_W, 0, 0, 1)*A.m(M_MU) + K[82]*A(F_W, 0, 0, 2)*A.m(M_LAM) + K[83]*A(F_W, 0, 0, 2)*A.m(M_MU) - K[84]*A(F_W, 0, 0, 3)*A.m(M_LAM) - K[85]*A(F_W, 0, 0, 3)*A.m(M_MU) - K[86]*A(F_W, 0, 0, -1)*A.m(M_LAM) - K[87]*A(F_W, 0, 0, -1)*A.m(M_MU) + K[88]*A(F_W, 0, 0, -2)*A.m(M_LAM) + K[89]*A(F_W, 0, 0, -2)*A.m(M_MU) - K[90]*A(F_W, 0, 0, -3)*A.m(M_LAM) - K[91]*A(F_W, 0, 0, -3)*A.m(M_MU) + K[92]*A(F_W, 0, 0, -4)*A.m(M_LAM) + K[93]*A(F_W, 0, 0, -4)*A.m(M_MU) + K[94]*A(F_W, 0, 0, 0)*A.m(M_LAM) + K[95]*A(F_W, 0, 0, 0)*A.m(M_MU);
    out[3] = A(F_TXY, 0, 0, 0) + K[96]*A(F_U, 0, 1, 0)*A.m(M_MU12) - K[97]*A(F_U, 0, 2, 0)*A.m(M_MU12) + K[98]*A(F_U, 0, 3, 0)*A.m(M_MU12) - K[99]*A(F_U, 0, 4, 0)*A.m(M_MU12) + K[100]*A(F_U, 0, -1, 0)*A.m(M_MU12) - K[101]*A(F_U, 0, -2, 0)*A.m(M_MU12) + K[102]*A(F_U, 0, -3, 0)*A.m(M_MU12) - K[103]*A(F_U, 0, 0, 0)*A.m(M_MU12) + K[104]*A(F_V, 1, 0, 0)*A.m(M_MU12) - K[105]*A(F_V, 2, 0, 0)*A.m(M_MU12) + K[106]*A(F_V, 3, 0, 0)*A.m(M_MU12) - K[107]*A(F_V, 4, 0, 0)*A.m(M_MU12) + K[108]*A(F_V, -1, 0, 0)*A.m(M_MU12) - K[109]*A(F_V, -2, 0, 0)*A.m(M_MU12) + K[110]*A(F_V, -3, 0, 0)*A.m(M_MU12) - K[111]*A(F_V, 0, 0, 0)*A.m(M_MU12);
    out[4] = A(F_TYZ, 0, 0, 0) + K[112]*A(F_V, 0, 0, 1)*A.m(M_MU23) - K[113]*A(F_V, 0, 0, 2)*A.m(M_MU23) + K[114]*A(F_V, 0, 0, 3)*A.m(M_MU23) - K[115]*A(F_V, 0, 0, 4)*A.m(M_MU23) + K[116]*A(F_V, 0, 0, -1)*A.m(M_MU23) - K[117]*A(F_V, 0, 0, -2)*A.m(M_MU23) + K[118]*A(F_V, 0, 0, -3)*A.m(M_MU23) - K[119]*A(F_V, 0, 0, 0)*A.m(M_MU23) + K[120]*A(F_W, 0, 1, 0)*A.m(M_MU23) - K[121]*A(F_W, 0, 2, 0)*A.m(M_MU23) + K[122]*A(F_W, 0, 3, 0)*A.m(M_MU23) - K[123]*A(F_W, 0, 4, 0)*A.m(M_MU23) + K[124]*A(F_W, 0, -1, 0)*A.m(M_MU23) - K[125]*A(F_W, 0, -2, 0)*A.m(M_MU23) + K[126]*A(F_W, 0, -3, 0)*A.m(M_MU23) - K[127]*A(F_W, 0, 0, 0)*A.m(M_MU23);
    out[5] = A(F_TXZ, 0, 0, 0) + K[128]*A(F_U, 0, 0, 1)*A.m(M_MU13) - K[129]*A(F_U, 0, 0, 2)*A.m(M_MU13) + K[130]*A(F_U, 0, 0, 3)*A.m(M_MU13) - K[131]*A(F_U, 0, 0, 4)*A.m(M_MU13) + K[132]*A(F_U, 0, 0, -1)*A.m(M_MU13) - K[133]*A(F_U, 0, 0, -2)*A.m(M_MU13) + K[134]*A(F_U, 0, 0, -3)*A.m(M_MU13) - K[135]*A(F_U, 0, 0, 0)*A.m(M_MU13) + K[136]*A(F_W, 1, 0, 0)*A.m(M_MU13) - K[137]*A(F_W, 2, 0, 0)*A.m(M_MU13) + K[138]*A(F_W, 3, 0, 0)*A.m(M_MU13) - K[139]*A(F_W, 4, 0, 0)*A.m(M_MU13) + K[140]*A(F_W, -1, 0, 0)*A.m(M_MU13) - K[141]*A(F_W, -2, 0, 0)*A.m(M_MU13) + K[142]*A(F_W, -3, 0, 0)*A.m(M_MU13) - K[143]*A(F_W, 0, 0, 0)*A.m(M_MU13);
  }
  template <typename C, class Acc, class KT>
  __device__ __forceinline__ static void velocity(const Acc &A, const KT &K, C out[3]) {
    out[0] = K[0]*A(F_TXX, 1, 0, 0)*A.m(M_B1) - K[1]*A(F_TXX, 2, 0, 0)*A.m(M_B1) + K[2]*A(F_TXX, 3, 0, 0)*A.m(M_B1) - K[3]*A(F_TXX, 4, 0, 0)*A.m(M_B1) + K[4]*A(F_TXX, -1, 0, 0)*A.m(M_B1) - K[5]*A(F_TXX, -2, 0, 0)*A.m(M_B1) + K[6]*A(F_TXX, -3, 0, 0)*A.m(M_B1) - K[7]*A(F_TXX, 0, 0, 0)*A.m(M_B1) - K[8]*A(F_TXY, 0, 1, 0)*A.m(M_B1) + K[9]*A(F_TXY, 0, 2, 0)*A.m(M_B1) - K[10]*A(F_TXY, 0, 3, 0)*A.m(M_B1) - K[11]*A(F_TXY, 0, -1, 0)*A.m(M_B1) + K[12]*A(F_TXY, 0, -2, 0)*A.m(M_B1) - K[13]*A(F_TXY, 0, -3, 0)*A.m(M_B1) + K[14]*A(F_TXY, 0, -4, 0)*A.m(M_B1) + K[15]*A(F_TXY, 0, 0, 0)*A.m(M_B1) - K[16]*A(F_TXZ, 0, 0, 1)*A.m(M_B1) + K[17]*A(F_TXZ, 0, 0, 2)*A.m(M_B1) - K[18]*A(F_TXZ, 0, 0, 3)*A.m(M_B1) - K[19]*A(F_TXZ, 0, 0, -1)*A.m(M_B1) + K[20]*A(F_TXZ, 0, 0, -2)*A.m(M_B1) - K[21]*A(F_TXZ, 0, 0, -3)*A.m(M_B1) + K[22]*A(F_TXZ, 0, 0, -4)*A.m(M_B1) + K[23]*A(F_TXZ, 0, 0, 0)*A.m(M_B1) + A(F_U, 0, 0, 0);
    out[1] = -K[24]*A(F_TXY, 1, 0, 0)*A.m(M_B2) + K[25]*A(F_TXY, 2, 0, 0)*A.m(M_B2) - K[26]*A(F_TXY, 3, 0, 0)*A.m(M_B2) - K[27]*A(F_TXY, -1, 0, 0)*A.m(M_B2) + K[28]*A(F_TXY, -2, 0, 0)*A.m(M_B2) - K[29]*A(F_TXY, -3, 0, 0)*A.m(M_B2) + K[30]*A(F_TXY, -4, 0, 0)*A.m(M_B2) + K[31]*A(F_TXY, 0, 0, 0)*A.m(M_B2) + K[32]*A(F_TYY, 0, 1, 0)*A.m(M_B2) - K[33]*A(F_TYY, 0, 2, 0)*A.m(M_B2) + K[34]*A(F_TYY, 0, 3, 0)*A.m(M_B2) - K[35]*A(F_TYY, 0, 4, 0)*A.m(M_B2) + K[36]*A(F_TYY, 0, -1, 0)*A.m(M_B2) - K[37]*A(F_TYY, 0, -2, 0)*A.m(M_B2) + K[38]*A(F_TYY, 0, -3, 0)*A.m(M_B2) - K[39]*A(F_TYY, 0, 0, 0)*A.m(M_B2) - K[40]*A(F_TYZ, 0, 0, 1)*A.m(M_B2) + K[41]*A(F_TYZ, 0, 0, 2)*A.m(M_B2) - K[42]*A(F_TYZ, 0, 0, 3)*A.m(M_B2) - K[43]*A(F_TYZ, 0, 0, -1)*A.m(M_B2) + K[44]*A(F_TYZ, 0, 0, -2)*A.m(M_B2) - K[45]*A(F_TYZ, 0, 0, -3)*A.m(M_B2) + K[46]*A(F_TYZ, 0, 0, -4)*A.m(M_B2) + K[47]*A(F_TYZ, 0, 0, 0)*A.m(M_B2) + A(F_V, 0, 0, 0);
    out[2] = -K[48]*A(F_TXZ, 1, 0, 0)*A.m(M_B3) + K[49]*A(F_TXZ, 2, 0, 0)*A.m(M_B3) - K[50]*A(F_TXZ, 3, 0, 0)*A.m(M_B3) - K[51]*A(F_TXZ, -1, 0, 0)*A.m(M_B3) + K[52]*A(F_TXZ, -2, 0, 0)*A.m(M_B3) - K[53]*A(F_TXZ, -3, 0, 0)*A.m(M_B3) + K[54]*A(F_TXZ, -4, 0, 0)*A.m(M_B3) + K[55]*A(F_TXZ, 0, 0, 0)*A.m(M_B3) - K[56]*A(F_TYZ, 0, 1, 0)*A.m(M_B3) + K[57]*A(F_TYZ, 0, 2, 0)*A.m(M_B3) - K[58]*A(F_TYZ, 0, 3, 0)*A.m(M_B3) - K[59]*A(F_TYZ, 0, -1, 0)*A.m(M_B3) + K[60]*A(F_TYZ, 0, -2, 0)*A.m(M_B3) - K[61]*A(F_TYZ, 0, -3, 0)*A.m(M_B3) + K[62]*A(F_TYZ, 0, -4, 0)*A.m(M_B3) + K[63]*A(F_TYZ, 0, 0, 0)*A.m(M_B3) + K[64]*A(F_TZZ, 0, 0, 1)*A.m(M_B3) - K[65]*A(F_TZZ, 0, 0, 2)*A.m(M_B3) + K[66]*A(F_TZZ, 0, 0, 3)*A.m(M_B3) - K[67]*A(F_TZZ, 0, 0, 4)*A.m(M_B3) + K[68]*A(F_TZZ, 0, 0, -1)*A.m(M_B3) - K[69]*A(F_TZZ, 0, 0, -2)*A.m(M_B3) + K[70]*A(F_TZZ, 0, 0, -3)*A.m(M_B3) - K[71]*A(F_TZZ, 0, 0, 0)*A.m(M_B3) + A(F_W, 0, 0, 0);
  }
};

// Literal index -> index among the distinct unit rationals of the
// heterogeneous expression (tables K_i = r_i dt / h repeat a few values).
template <int R, bool STRESS> struct KMap { static constexpr bool ok = false; };

template <> struct KMap<1, true> {
  static constexpr bool ok = true;
  static constexpr int NU = 2, NK = 36;
  __host__ __device__ static constexpr int at(int i) {
    constexpr int m[36] = {0, 1, 0, 1, 0, 0, 0, 0, 0, 0, 0, 1, 0, 1, 0, 0, 0, 0, 0, 0, 0, 1, 0, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    return m[i];
  }
};

template <> struct KMap<1, false> {
  static constexpr bool ok = true;
  static constexpr int NU = 1, NK = 18;
  __host__ __device__ static constexpr int at(int i) {
    constexpr int m[18] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    return m[i];
  }
};

template <> struct KMap<2, true> {
  static constexpr bool ok = true;
  static constexpr int NU = 4, NK = 72;
  __host__ __device__ static constexpr int at(int i) {
    constexpr int m[72] = {0, 1, 2, 3, 0, 1, 2, 3, 0, 2, 0, 2, 0, 2, 0, 2, 0, 2, 0, 2, 0, 1, 2, 3, 0, 1, 2, 3, 0, 2, 0, 2, 0, 2, 0, 2, 0, 2, 0, 2, 0, 1, 2, 3, 0, 1, 2, 3, 2, 0, 0, 2, 2, 0, 0, 2, 2, 0, 0, 2, 2, 0, 0, 2, 2, 0, 0, 2, 2, 0, 0, 2};
    return m[i];
  }
};

template <> struct KMap<2, false> {
  static constexpr bool ok = true;
  static constexpr int NU = 2, NK = 36;
  __host__ __device__ static constexpr int at(int i) {
    constexpr int m[36] = {0, 1, 1, 0, 1, 0, 1, 0, 1, 0, 1, 0, 1, 0, 1, 0, 0, 1, 1, 0, 1, 0, 1, 0, 1, 0, 1, 0, 1, 0, 1, 0, 0, 1, 1, 0};
    return m[i];
  }
};

template <> struct KMap<3, true> {
  static constexpr bool ok = true;
  static constexpr int NU = 6, NK = 108;
  __host__ __device__ static constexpr int at(int i) {
    constexpr int m[108] = {0, 1, 2, 3, 4, 5, 0, 1, 2, 3, 4, 5, 0, 2, 4, 0, 2, 4, 0, 2, 4, 0, 2, 4, 0, 2, 4, 0, 2, 4, 0, 1, 2, 3, 4, 5, 0, 1, 2, 3, 4, 5, 0, 2, 4, 0, 2, 4, 0, 2, 4, 0, 2, 4, 0, 2, 4, 0, 2, 4, 0, 1, 2, 3, 4, 5, 0, 1, 2, 3, 4, 5, 4, 0, 2, 0, 2, 4, 4, 0, 2, 0, 2, 4, 4, 0, 2, 0, 2, 4, 4, 0, 2, 0, 2, 4, 4, 0, 2, 0, 2, 4, 4, 0, 2, 0, 2, 4};
    return m[i];
  }
};

template <> struct KMap<3, false> {
  static constexpr bool ok = true;
  static constexpr int NU = 3, NK = 54;
  __host__ __device__ static constexpr int at(int i) {
    constexpr int m[54] = {0, 1, 2, 1, 2, 0, 1, 2, 0, 1, 2, 0, 1, 2, 0, 1, 2, 0, 1, 2, 0, 1, 2, 0, 0, 1, 2, 1, 2, 0, 1, 2, 0, 1, 2, 0, 1, 2, 0, 1, 2, 0, 1, 2, 0, 1, 2, 0, 0, 1, 2, 1, 2, 0};
    return m[i];
  }
};

template <> struct KMap<4, true> {
  static constexpr bool ok = true;
  static constexpr int NU = 8, NK = 144;
  __host__ __device__ static constexpr int at(int i) {
    constexpr int m[144] = {0, 1, 2, 3, 4, 5, 6, 7, 0, 1, 2, 3, 4, 5, 6, 7, 0, 2, 4, 6, 0, 2, 4, 6, 0, 2, 4, 6, 0, 2, 4, 6, 0, 2, 4, 6, 0, 2, 4, 6, 0, 1, 2, 3, 4, 5, 6, 7, 0, 1, 2, 3, 4, 5, 6, 7, 0, 2, 4, 6, 0, 2, 4, 6, 0, 2, 4, 6, 0, 2, 4, 6, 0, 2, 4, 6, 0, 2, 4, 6, 0, 1, 2, 3, 4, 5, 6, 7, 0, 1, 2, 3, 4, 5, 6, 7, 6, 0, 2, 4, 0, 2, 4, 6, 6, 0, 2, 4, 0, 2, 4, 6, 6, 0, 2, 4, 0, 2, 4, 6, 6, 0, 2, 4, 0, 2, 4, 6, 6, 0, 2, 4, 0, 2, 4, 6, 6, 0, 2, 4, 0, 2, 4, 6};
    return m[i];
  }
};

template <> struct KMap<4, false> {
  static constexpr bool ok = true;
  static constexpr int NU = 4, NK = 72;
  __host__ __device__ static constexpr int at(int i) {
    constexpr int m[72] = {0, 1, 2, 3, 1, 2, 3, 0, 1, 2, 3, 0, 1, 2, 3, 0, 1, 2, 3, 0, 1, 2, 3, 0, 1, 2, 3, 0, 1, 2, 3, 0, 0, 1, 2, 3, 1, 2, 3, 0, 1, 2, 3, 0, 1, 2, 3, 0, 1, 2, 3, 0, 1, 2, 3, 0, 1, 2, 3, 0, 1, 2, 3, 0, 0, 1, 2, 3, 1, 2, 3, 0};
    return m[i];
  }
};

}  // namespace ofd
