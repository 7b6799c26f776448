// VTK XML structured-grid (.vts) output of one host field, the library form
// of opesci_dump_field_vts_3d (src/opesciIO.cpp:614-667), which the
// reference's generated code calls after every step when output_vts is set
// (opesci/regulargrid.py:702-719).  The reference writes through VTK with a
// zlib compressor; VTK is not a dependency here, so the file is written
// directly in the same format with the data appended raw (uncompressed):
// a UInt64 byte count before each array, little-endian Float32 values.  The
// points follow the reference's insertion order (x outer, z inner) with
// coordinates (index - margin) * spacing rounded to float, and the one
// point-data array "field" holds the values in memory order.
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "ofd.h"

namespace ofd {
int fail_msg(int code, const char *msg);
}

namespace {

bool put_block(FILE *fp, const float *data, uint64_t count) {
  const uint64_t nbytes = count * sizeof(float);
  return fwrite(&nbytes, sizeof(nbytes), 1, fp) == 1 && (count == 0 || fwrite(data, sizeof(float), count, fp) == count);
}

}  // namespace

extern "C" int ofd_write_field_vts_3d(const char *name, const int dims[3], const float spacing[3], int margin,
                                      const float *field) {
  if (!name || !dims || !spacing || !field) return ofd::fail_msg(OFD_EINVAL, "null argument");
  if (dims[0] <= 0 || dims[1] <= 0 || dims[2] <= 0) return ofd::fail_msg(OFD_EINVAL, "dims must be positive");
  const uint64_t n = (uint64_t)dims[0] * dims[1] * dims[2];
  std::vector<float> pts;
  pts.reserve(3 * n);
  for (int i = 0; i < dims[0]; ++i) {
    const float x = (i - margin) * spacing[0];
    for (int j = 0; j < dims[1]; ++j) {
      const float y = (j - margin) * spacing[1];
      for (int k = 0; k < dims[2]; ++k) {
        pts.push_back(x);
        pts.push_back(y);
        pts.push_back((k - margin) * spacing[2]);
      }
    }
  }
  const std::string path = std::string(name) + ".vts";
  FILE *fp = fopen(path.c_str(), "wb");
  if (!fp) return ofd::fail_msg(OFD_EINVAL, ("cannot open " + path + " for writing").c_str());
  const unsigned long long off_points = sizeof(uint64_t) + n * sizeof(float);
  const int ex = dims[0] - 1, ey = dims[1] - 1, ez = dims[2] - 1;
  fprintf(fp,
          "<?xml version=\"1.0\"?>\n"
          "<VTKFile type=\"StructuredGrid\" version=\"1.0\" byte_order=\"LittleEndian\" header_type=\"UInt64\">\n"
          "  <StructuredGrid WholeExtent=\"0 %d 0 %d 0 %d\">\n"
          "    <Piece Extent=\"0 %d 0 %d 0 %d\">\n"
          "      <PointData>\n"
          "        <DataArray type=\"Float32\" Name=\"field\" NumberOfComponents=\"1\" format=\"appended\" "
          "offset=\"0\"/>\n"
          "      </PointData>\n"
          "      <Points>\n"
          "        <DataArray type=\"Float32\" Name=\"Points\" NumberOfComponents=\"3\" format=\"appended\" "
          "offset=\"%llu\"/>\n"
          "      </Points>\n"
          "    </Piece>\n"
          "  </StructuredGrid>\n"
          "  <AppendedData encoding=\"raw\">\n"
          "_",
          ex, ey, ez, ex, ey, ez, off_points);
  bool ok = put_block(fp, field, n) && put_block(fp, pts.data(), 3 * n);
  ok = ok && fputs("\n  </AppendedData>\n</VTKFile>\n", fp) >= 0;
  ok = (fclose(fp) == 0) && ok;
  if (!ok) return ofd::fail_msg(OFD_EINVAL, ("short write to " + path).c_str());
  return OFD_OK;
}
