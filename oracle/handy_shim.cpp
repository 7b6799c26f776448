// ORACLE build helper (test infrastructure only): C entry points over the
// reference's own trace resampling, opesci_resample_timeseries
// (src/opesciHandy.cpp:125-195), and SEG-Y model reader,
// opesci_read_model_segy (src/opesciIO.cpp:419-612), so that fixture scripts
// can call them through ctypes.  Compiled together with the reference's
// src/opesciHandy.cpp and src/opesciIO.cpp (without VTK) into
// oracle/_ref/libopescihandy.so by oracle/Makefile.
#include <vector>

#include "opesciHandy.h"
#include "opesciIO.h"

extern "C" int ref_resample_timeseries(const float *src, int n, float dt, double sdt, float *out, int cap) {
  std::vector<float> in(src, src + n), res;
  opesci_resample_timeseries(in, dt, sdt, res);
  const int m = (int)res.size();
  for (int i = 0; i < m && i < cap; ++i) out[i] = res[i];
  return m;
}

extern "C" int ref_read_model_segy(const char *path, float *out, long cap, int dim[3], float spacing[3]) {
  std::vector<float> a;
  if (opesci_read_model_segy(path, a, dim, spacing)) return -1;
  for (long i = 0; i < (long)a.size() && i < cap; ++i) out[i] = a[i];
  return (int)a.size();
}
