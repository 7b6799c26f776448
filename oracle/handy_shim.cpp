// ORACLE build helper (test infrastructure only): a C entry point over the
// reference's own trace resampling, opesci_resample_timeseries
// (src/opesciHandy.cpp:125-195), so that fixture scripts can call it through
// ctypes.  Compiled together with the reference's src/opesciHandy.cpp into
// oracle/_ref/libopescihandy.so by oracle/Makefile.
#include <vector>

#include "opesciHandy.h"

extern "C" int ref_resample_timeseries(const float *src, int n, float dt, double sdt, float *out, int cap) {
  std::vector<float> in(src, src + n), res;
  opesci_resample_timeseries(in, dt, sdt, res);
  const int m = (int)res.size();
  for (int i = 0; i < m && i < cap; ++i) out[i] = res[i];
  return m;
}
