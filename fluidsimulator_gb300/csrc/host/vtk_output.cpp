// Frame output of particle positions as VTK PolyData (.vtp) and a ParaView
// time series (.pvd).
//
// ASCII output reproduces the reference's VtkWriter byte for byte
// (io/src/vtk_writer.cpp:25-79: 9 fixed decimals, one vertex per point) so
// existing tooling keeps working. Binary output writes the same PolyData
// with an appended raw block (UInt64 size headers): 20 bytes per particle
// instead of ~55 bytes of text, and no float formatting.

#include <cinttypes>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "fluid_gb300.h"

namespace {

bool write_ascii(FILE* f, const float* x, const float* y, const float* z, int64_t n) {
  std::fprintf(f, "<?xml version=\"1.0\"?>\n");
  std::fprintf(f, "<VTKFile type=\"PolyData\" version=\"0.1\" byte_order=\"LittleEndian\">\n");
  std::fprintf(f, "  <PolyData>\n");
  std::fprintf(f,
               "    <Piece NumberOfPoints=\"%" PRId64 "\" NumberOfVerts=\"%" PRId64
               "\" NumberOfLines=\"0\" NumberOfStrips=\"0\" NumberOfPolys=\"0\">\n",
               n, n);
  std::fprintf(f, "      <Points>\n");
  std::fprintf(f, "        <DataArray type=\"Float32\" NumberOfComponents=\"3\" format=\"ascii\">\n");
  for (int64_t i = 0; i < n; ++i)
    std::fprintf(f, "          %.9f %.9f %.9f\n", static_cast<double>(x[i]), static_cast<double>(y[i]),
                 static_cast<double>(z[i]));
  std::fprintf(f, "        </DataArray>\n      </Points>\n      <Verts>\n");
  std::fprintf(f, "        <DataArray type=\"Int32\" Name=\"connectivity\" format=\"ascii\">\n");
  for (int64_t i = 0; i < n; ++i) std::fprintf(f, "          %" PRId64 "\n", i);
  std::fprintf(f, "        </DataArray>\n");
  std::fprintf(f, "        <DataArray type=\"Int32\" Name=\"offsets\" format=\"ascii\">\n");
  for (int64_t i = 0; i < n; ++i) std::fprintf(f, "          %" PRId64 "\n", i + 1);
  std::fprintf(f, "        </DataArray>\n      </Verts>\n    </Piece>\n  </PolyData>\n</VTKFile>\n");
  return !std::ferror(f);
}

bool write_binary(FILE* f, const float* x, const float* y, const float* z, int64_t n) {
  const uint64_t pts = 12ull * static_cast<uint64_t>(n), ints = 4ull * static_cast<uint64_t>(n);
  const uint64_t off_conn = 8 + pts, off_offs = off_conn + 8 + ints;
  std::fprintf(f, "<?xml version=\"1.0\"?>\n");
  std::fprintf(f,
               "<VTKFile type=\"PolyData\" version=\"0.1\" byte_order=\"LittleEndian\" "
               "header_type=\"UInt64\">\n");
  std::fprintf(f, "  <PolyData>\n");
  std::fprintf(f,
               "    <Piece NumberOfPoints=\"%" PRId64 "\" NumberOfVerts=\"%" PRId64
               "\" NumberOfLines=\"0\" NumberOfStrips=\"0\" NumberOfPolys=\"0\">\n",
               n, n);
  std::fprintf(f,
               "      <Points>\n        <DataArray type=\"Float32\" NumberOfComponents=\"3\" "
               "format=\"appended\" offset=\"0\"/>\n      </Points>\n");
  std::fprintf(f,
               "      <Verts>\n        <DataArray type=\"Int32\" Name=\"connectivity\" format=\"appended\" "
               "offset=\"%" PRIu64 "\"/>\n",
               off_conn);
  std::fprintf(f,
               "        <DataArray type=\"Int32\" Name=\"offsets\" format=\"appended\" offset=\"%" PRIu64
               "\"/>\n      </Verts>\n",
               off_offs);
  std::fprintf(f, "    </Piece>\n  </PolyData>\n  <AppendedData encoding=\"raw\">\n   _");
  const int64_t chunk = 1 << 16;
  std::vector<float> xyz(3 * static_cast<size_t>(chunk < n ? chunk : (n > 0 ? n : 1)));
  std::vector<int32_t> iv(static_cast<size_t>(chunk < n ? chunk : (n > 0 ? n : 1)));
  std::fwrite(&pts, sizeof(pts), 1, f);
  for (int64_t s = 0; s < n; s += chunk) {
    const int64_t m = (n - s < chunk) ? n - s : chunk;
    for (int64_t k = 0; k < m; ++k) {
      xyz[3 * k] = x[s + k];
      xyz[3 * k + 1] = y[s + k];
      xyz[3 * k + 2] = z[s + k];
    }
    std::fwrite(xyz.data(), sizeof(float), static_cast<size_t>(3 * m), f);
  }
  for (int pass = 0; pass < 2; ++pass) {
    std::fwrite(&ints, sizeof(ints), 1, f);
    for (int64_t s = 0; s < n; s += chunk) {
      const int64_t m = (n - s < chunk) ? n - s : chunk;
      for (int64_t k = 0; k < m; ++k) iv[k] = static_cast<int32_t>(s + k + pass);
      std::fwrite(iv.data(), sizeof(int32_t), static_cast<size_t>(m), f);
    }
  }
  std::fprintf(f, "\n  </AppendedData>\n</VTKFile>\n");
  return !std::ferror(f);
}

}  // namespace

extern "C" int fluid_write_vtp(const char* path, const float* pos_x, const float* pos_y, const float* pos_z,
                               int64_t count, int32_t binary) {
  if (!path || count < 0 || (count > 0 && (!pos_x || !pos_y || !pos_z))) return FLUID_ERR_INVALID_ARGUMENT;
  FILE* f = std::fopen(path, binary ? "wb" : "w");
  if (!f) return FLUID_ERR_INVALID_ARGUMENT;
  const bool ok = binary ? write_binary(f, pos_x, pos_y, pos_z, count) : write_ascii(f, pos_x, pos_y, pos_z, count);
  const bool closed = std::fclose(f) == 0;
  return (ok && closed) ? FLUID_OK : FLUID_ERR_INVALID_ARGUMENT;
}

extern "C" int fluid_write_pvd(const char* path, const double* times, const char* const* files, int64_t count) {
  if (!path || count < 0 || (count > 0 && (!times || !files))) return FLUID_ERR_INVALID_ARGUMENT;
  FILE* f = std::fopen(path, "w");
  if (!f) return FLUID_ERR_INVALID_ARGUMENT;
  std::fprintf(f, "<?xml version=\"1.0\"?>\n");
  std::fprintf(f, "<VTKFile type=\"Collection\" version=\"0.1\" byte_order=\"LittleEndian\">\n");
  std::fprintf(f, "  <Collection>\n");
  for (int64_t k = 0; k < count; ++k)
    std::fprintf(f, "    <DataSet timestep=\"%.9f\" group=\"\" part=\"0\" file=\"%s\"/>\n", times[k], files[k]);
  std::fprintf(f, "  </Collection>\n</VTKFile>\n");
  const bool ok = !std::ferror(f);
  return (std::fclose(f) == 0 && ok) ? FLUID_OK : FLUID_ERR_INVALID_ARGUMENT;
}
