// Drives the drop-in shim the way the reference's application does
// (app/src/main.cpp:171-184 device check, :250-251 one fluid::cuda_step per
// step, then reads state.pos_* / state.time), on a scene read from a file.
// Usage: shim_app_main <in.bin> <out.bin> <steps>
// in.bin : raw fluid_params, int64 count, then pos_x..vel_z (count floats each)
// out.bin: pos_x..vel_z after <steps> steps, then float time.
// Like the reference's main, it calls cuda_step outside any try block.
#include <cstdio>
#include <iostream>
#include <vector>

#include "fluid/cuda.h"
#include "fluid_gb300.h"

int main(int argc, char** argv) {
  if (argc != 4) return 2;
  int device_count = 0;
  const char* cuda_error = nullptr;
  if (!fluid::cuda_device_available(&device_count, &cuda_error)) {
    std::cerr << "CUDA backend unavailable: " << (cuda_error ? cuda_error : "no CUDA devices detected.") << std::endl;
    return 1;
  }
  std::cout << "backend=cuda" << std::endl << "cuda_devices=" << device_count << std::endl;
  FILE* in = std::fopen(argv[1], "rb");
  if (!in) return 3;
  fluid_params cp;
  int64_t n = 0;
  if (std::fread(&cp, sizeof(cp), 1, in) != 1 || std::fread(&n, sizeof(n), 1, in) != 1) return 3;
  fluid::State st;
  std::vector<float>* arr[6] = {&st.pos_x, &st.pos_y, &st.pos_z, &st.vel_x, &st.vel_y, &st.vel_z};
  for (auto* a : arr) {
    a->resize(static_cast<std::size_t>(n));
    if (std::fread(a->data(), sizeof(float), a->size(), in) != a->size()) return 3;
  }
  std::fclose(in);
  fluid::Params p;
  p.dt = cp.dt;
  p.density = cp.density;
  p.particle_mass = cp.particle_mass;
  p.h = cp.h;
  p.particle_radius = cp.particle_radius;
  p.epsilon = cp.epsilon;
  p.solver_iterations = cp.solver_iterations;
  p.neighbor_reserve_factor = cp.neighbor_reserve_factor;
  p.use_uniform_grid = cp.use_uniform_grid != 0;
  p.enable_scorr = cp.enable_scorr != 0;
  p.enable_xsph = cp.enable_xsph != 0;
  p.enable_vorticity = cp.enable_vorticity != 0;
  p.scorr_k = cp.scorr_k;
  p.scorr_n = cp.scorr_n;
  p.scorr_dq_coeff = cp.scorr_dq_coeff;
  p.visc_c = cp.visc_c;
  p.plane_restitution = cp.plane_restitution;
  p.plane_friction = cp.plane_friction;
  p.vort_epsilon = cp.vort_epsilon;
  p.vort_norm_eps = cp.vort_norm_eps;
  p.external_forces.x = cp.external_force[0];
  p.external_forces.y = cp.external_force[1];
  p.external_forces.z = cp.external_force[2];
  for (int q = 0; q < cp.plane_count; ++q) p.planes.add(cp.plane_nx[q], cp.plane_ny[q], cp.plane_nz[q], cp.plane_d[q]);
  const int steps = std::atoi(argv[3]);
  for (int s = 0; s < steps; ++s) fluid::cuda_step(p, st);
  FILE* out = std::fopen(argv[2], "wb");
  if (!out) return 4;
  for (auto* a : arr) std::fwrite(a->data(), sizeof(float), a->size(), out);
  std::fwrite(&st.time, sizeof(float), 1, out);
  std::fclose(out);
  std::cout << "particle_count=" << st.size() << std::endl;
  return 0;
}
