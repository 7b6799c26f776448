// Correctly rounded double quotients x / D of many numerators sharing one
// divisor, at a fraction of the FP64 work of one IEEE division each.
//
// Method (Markstein, "Computation of elementary functions on the IBM RISC
// System/6000 processor", IBM J. Res. Develop. 34(1), 1990; restated in
// Muller et al., "Handbook of Floating-Point Arithmetic", the theorem on
// division by FMA correction): if y = RN(1/D) and q is within one ulp of
// x / D, then the remainder r = x - D q is exactly representable (one FMA
// computes it exactly) and RN(q + r y) = RN(x / D).
//
// y is CUDA's correctly rounded reciprocal (__drcp_rn).  q0 = RN(x y) carries
// the errors of y and of one rounding, so it can sit slightly more than one
// ulp away from x / D; one refinement q1 = RN(q0 + RN(x - D q0) y) brings it
// within half an ulp plus a term of order 2^-52 ulp, after which the
// correction step above applies.  Per quotient: one multiply and four FMAs.
//
// The theorem assumes no overflow or underflow in the remainders: operands
// outside [2^-400, 2^400] in magnitude (zeros, infinities, NaNs, a zero or
// huge divisor) take the plain IEEE division, so every input gives x / D.
#pragma once

namespace ofd {

struct SharedDiv {
  double D, y;
  bool ok;
  __device__ __forceinline__ explicit SharedDiv(float Df) : D((double)Df) {
    const double ad = fabs(D);
    ok = ad > 0x1p-400 && ad < 0x1p400;
    y = ok ? __drcp_rn(D) : 0.0;
  }
  __device__ __forceinline__ double div(double x) const {
    const double ax = fabs(x);
    if (!ok || !(ax > 0x1p-400 && ax < 0x1p400)) return x / D;
    double q = x * y;
    double r = fma(-D, q, x);
    q = fma(r, y, q);
    r = fma(-D, q, x);
    return fma(r, y, q);
  }
};

}  // namespace ofd
