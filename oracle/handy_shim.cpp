// ORACLE build helper (test infrastructure only): C entry points over the
// reference's own trace resampling, opesci_resample_timeseries
// (src/opesciHandy.cpp:125-195), SEG-Y model reader, opesci_read_model_segy
// (src/opesciIO.cpp:419-612), source and receiver file readers
// (src/opesciIO.cpp:345-396), Lame constants and time step
// (src/opesciHandy.cpp:53-89), so that fixture scripts can call them through
// ctypes.  Compiled together with the reference's
// src/opesciHandy.cpp and src/opesciIO.cpp (without VTK) into
// oracle/_ref/libopescihandy.so by oracle/Makefile.
#include <cmath>
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

// opesci_read_receivers (src/opesciIO.cpp:374-396): the coordinates, up to
// cap floats; returns how many the file gave, -1 on failure.
extern "C" int ref_read_receivers(const char *path, float *out, int cap) {
  std::vector<float> a;
  if (opesci_read_receivers(path, a)) return -1;
  for (int i = 0; i < (int)a.size() && i < cap; ++i) out[i] = a[i];
  return (int)a.size();
}

// opesci_read_souces (src/opesciIO.cpp:345-372): coordinates into xyz and
// the three signals into sig (x, then y, then z), counts[0..3] their sizes.
extern "C" int ref_read_sources(const char *xyz_path, const char *xs, const char *ys, const char *zs, float *xyz,
                                int cap_xyz, float *sig, int cap_sig, int counts[4]) {
  std::vector<float> a, x, y, z;
  if (opesci_read_souces(xyz_path, xs, ys, zs, a, x, y, z)) return -1;
  for (int i = 0; i < (int)a.size() && i < cap_xyz; ++i) xyz[i] = a[i];
  int k = 0;
  for (const std::vector<float> *v : {&x, &y, &z})
    for (float f : *v)
      if (k < cap_sig) sig[k++] = f;
  counts[0] = (int)a.size();
  counts[1] = (int)x.size();
  counts[2] = (int)y.size();
  counts[3] = (int)z.size();
  return 0;
}

// opesci_calculate_lame_costants (src/opesciHandy.cpp:53-67)
extern "C" void ref_lame_constants(const float *vp, const float *vs, const float *rho, long n, float *mu, float *lam) {
  std::vector<float> a(vp, vp + n), b(vs, vs + n), c(rho, rho + n), m, l;
  opesci_calculate_lame_costants(a, b, c, m, l);
  for (long i = 0; i < n; ++i) {
    mu[i] = m[i];
    lam[i] = l[i];
  }
}

// opesci_calculate_dt (src/opesciHandy.cpp:69-89)
extern "C" float ref_calculate_dt(const float *vp, long n, float h) {
  std::vector<float> a(vp, vp + n);
  return opesci_calculate_dt(a, h);
}

// The index of a point at coordinate coor as the reference driver forms it
// for receivers and the source (tests/src/test_ref_iso_elastic.cpp:230-232,
// 277-279): (int)round(coor/h) with float operands.  The driver is a program
// with its own main, so its one-line formula is restated here.
extern "C" void ref_point_indices(const float *coor, long n, float h, int *out) {
  for (long i = 0; i < n; ++i) out[i] = (int)round(coor[i] / h);
}
