// Device self-checks of arithmetic helpers against CUDA's IEEE operations.
#include <cuda_runtime.h>
#include <cstdint>
#include "ofd.h"
#include "ofd_shared_div.cuh"

namespace {

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

// a double with the given exponent (unbiased) and random 52-bit mantissa
__device__ __forceinline__ double with_exp(uint64_t bits, int e) {
  const uint64_t m = bits & 0xFFFFFFFFFFFFFULL;
  return __longlong_as_double((long long)(((uint64_t)(e + 1023) << 52) | m));
}

// Operand pair i: D a float-valued divisor (the generated ghosts divide by a
// float), x of one of three kinds: random (exponents in +-60 around D's),
// near-exact (x = RN(q D) for a random q) and near-midpoint (below).  Signs
// random; a few zeros of either sign.
__global__ void shared_div_check_kernel(long n, uint64_t seed, unsigned long long *bad) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const uint64_t r0 = mix64(seed ^ (uint64_t)i * 0x2545F4914F6CDD1DULL);
    const uint64_t r1 = mix64(r0), r2 = mix64(r1), r3 = mix64(r2);
    const int ed = (int)(r3 % 61) - 30;
    const float Df = (float)with_exp(r1, ed) * ((r3 >> 8) & 1 ? -1.f : 1.f);
    const double D = (double)Df;
    const int kind = (int)((r3 >> 9) % 3);
    double x;
    if (kind == 0) {
      x = with_exp(r2, ed + (int)((r3 >> 12) % 121) - 60);
    } else {
      const double q = with_exp(r2, (int)((r3 >> 12) % 81) - 40);
      if (kind == 1) {
        x = q * D;
      } else {
        // x = RN((q + h) D), h half an ulp of q: x / D lies within about an
        // ulp of the midpoint between q and its successor (a quotient of two
        // binary floating-point numbers is never exactly a midpoint)
        const double up = __longlong_as_double(__double_as_longlong(q) + 1);
        x = fma(q, D, (up - q) * 0.5 * D);
      }
    }
    if ((r3 >> 20) % 4096 == 0) x = ((r3 >> 32) & 1) ? -0.0 : 0.0;
    if ((r3 >> 33) & 1) x = -x;
    const ofd::SharedDiv s(Df);
    const double a = s.div(x), b = x / D;
    if (__double_as_longlong(a) != __double_as_longlong(b) && !(a != a && b != b)) atomicAdd(bad, 1ULL);
  }
}

}  // namespace

extern "C" int ofd_check_shared_division(long n, unsigned long long seed, long *mismatches) {
  if (n < 0 || !mismatches) return OFD_EINVAL;
  unsigned long long *d = nullptr;
  if (cudaMalloc((void **)&d, sizeof(*d)) != cudaSuccess) return OFD_ECUDA;
  cudaMemset(d, 0, sizeof(*d));
  shared_div_check_kernel<<<1216, 256>>>(n, seed, d);
  unsigned long long h = 0;
  const cudaError_t e = cudaMemcpy(&h, d, sizeof(h), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess || cudaGetLastError() != cudaSuccess) return OFD_ECUDA;
  *mismatches = (long)h;
  return OFD_OK;
}
