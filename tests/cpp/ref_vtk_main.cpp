// Writes one frame and a two-entry series with the reference's VtkWriter /
// PvdWriter (io/src/vtk_writer.cpp), for the byte-for-byte output test.
// Usage: ref_vtk_main <positions.bin> <out_dir>   (int64 n, then x, y, z blocks)
#include <cstdio>
#include <vector>

#include "fluid/vtk_writer.h"

int main(int argc, char** argv) {
  if (argc != 3) return 2;
  FILE* f = std::fopen(argv[1], "rb");
  long long n = 0;
  if (!f || std::fread(&n, sizeof(n), 1, f) != 1) return 3;
  std::vector<float> p(3 * static_cast<size_t>(n));
  if (std::fread(p.data(), sizeof(float), p.size(), f) != p.size()) return 3;
  std::fclose(f);
  fluid::VtkWriter w(argv[2], "frame");
  fluid::VtkFrameView v;
  v.pos_x = p.data();
  v.pos_y = p.data() + n;
  v.pos_z = p.data() + 2 * n;
  v.count = static_cast<std::size_t>(n);
  if (!w.write_frame(v, 0)) return 4;
  fluid::PvdWriter pvd(argv[2], "series");
  pvd.add_frame(0.008333333, fluid::VtkWriter::make_frame_filename("frame", 0));
  pvd.add_frame(1.25, fluid::VtkWriter::make_frame_filename("frame", 1));
  return pvd.write() ? 0 : 5;
}
