// SEG-Y model decoding on the device: the IBM-float samples of a whole
// format-1 SEG-Y image (the reference reads them one by one on the host,
// src/opesciIO.cpp:400-417,586-603) turned into the model array
// out[iz][iy][ix] in one pass.  Consecutive threads take consecutive samples
// of a trace, so reads are contiguous; each sample lands at its model index.
#include <cstdint>

namespace {

// +-mantissa / 2^24 * 16^(exponent - 64), sign applied to the integer
// mantissa, in double (exact: a 24-bit integer times a power of two within
// the double range), rounded to float.
__device__ __forceinline__ float ibm_word_to_float(uint32_t w) {
  const int e = (int)((w >> 24) & 0x7f) - 64;
  const long long mant = (long long)(w & 0xffffff);
  const long long sm = (w >> 31) ? -mant : mant;
  const double v = ((double)sm / 16777216.0) * ldexp(1.0, 4 * e);
  return __double2float_rn(v);
}

__global__ void segy_ibm_decode_kernel(const unsigned char *__restrict__ file, long tracesize, int nx, int ny,
                                       int nz, int swap, float *__restrict__ out) {
  const long n = (long)nx * ny * nz;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const long tr = i / nz;
    const int iz = (int)(i - tr * nz);
    const unsigned char *p = file + 3600 + tr * tracesize + 240 + 4L * iz;
    // the reference reads the four bytes (swapped when the header was) as a
    // little-endian word
    const uint32_t w = swap ? ((uint32_t)p[0] << 24 | (uint32_t)p[1] << 16 | (uint32_t)p[2] << 8 | p[3])
                            : ((uint32_t)p[3] << 24 | (uint32_t)p[2] << 16 | (uint32_t)p[1] << 8 | p[0]);
    const int ix = (int)(tr % nx), iy = (int)(tr / nx);
    out[ix + (long)iy * nx + (long)iz * nx * ny] = ibm_word_to_float(w);
  }
}

}  // namespace

namespace ofd {

// Decode a SEG-Y image (host memory, file_size >= 3600 + nx*ny*(240+4*nz)
// checked by the caller) into out (host, nz*ny*nx floats).
cudaError_t segy_decode(const void *file, long file_size, int nx, int ny, int nz, int swap, float *out) {
  const long tracesize = 240 + 4L * nz;
  const long need = 3600 + (long)nx * ny * tracesize;
  unsigned char *d_file = nullptr;
  float *d_out = nullptr;
  const size_t nbytes = sizeof(float) * (size_t)nx * ny * nz;
  cudaStream_t st = nullptr;
  cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMallocAsync((void **)&d_file, (size_t)need, st);
  if (e == cudaSuccess) e = cudaMallocAsync((void **)&d_out, nbytes, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_file, file, (size_t)need, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) {
    segy_ibm_decode_kernel<<<1216, 256, 0, st>>>(d_file, tracesize, nx, ny, nz, swap ? 1 : 0, d_out);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, d_out, nbytes, cudaMemcpyDeviceToHost, st);
  if (d_file) cudaFreeAsync(d_file, st);
  if (d_out) cudaFreeAsync(d_out, st);
  if (st) {
    const cudaError_t e2 = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = e2;
    cudaStreamDestroy(st);
  }
  (void)file_size;
  return e;
}

}  // namespace ofd
