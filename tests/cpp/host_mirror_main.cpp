// Test driver for the C++ host interface (fluidsimulator_gb300/csrc/host).
// Usage: host_mirror_main <in.bin> <out.bin> <steps> <cuda_step|solver>
// in.bin : raw fluid_params, int64 count, then pos_x..vel_z (count floats each)
// out.bin: pos_x..vel_z after <steps> steps, then float time.
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "fluid_gb300.hpp"

int main(int argc, char** argv) {
  if (argc != 5) return 2;
  FILE* in = std::fopen(argv[1], "rb");
  if (!in) return 3;
  fluid_params cp;
  int64_t n = 0;
  if (std::fread(&cp, sizeof(cp), 1, in) != 1 || std::fread(&n, sizeof(n), 1, in) != 1) return 3;
  fluid_gb300::State st = fluid_gb300::make_state(static_cast<std::size_t>(n));
  std::vector<float>* arr[6] = {&st.pos_x, &st.pos_y, &st.pos_z, &st.vel_x, &st.vel_y, &st.vel_z};
  for (auto* a : arr)
    if (std::fread(a->data(), sizeof(float), static_cast<std::size_t>(n), in) != static_cast<std::size_t>(n)) return 3;
  std::fclose(in);

  fluid_gb300::Params p;  // rebuilt field by field through the mirror type
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
  if (cp.plane_friction_per_plane) p.plane_friction_each.assign(cp.plane_friction_each, cp.plane_friction_each + cp.plane_count);

  int count = 0;
  const char* err = nullptr;
  if (!fluid_gb300::cuda_device_available(&count, &err)) {
    std::fprintf(stderr, "no device: %s\n", err ? err : "none");
    return 4;
  }
  const int steps = std::stoi(argv[3]);
  try {
    if (std::string(argv[4]) == "cuda_step") {
      for (int k = 0; k < steps; ++k) fluid_gb300::cuda_step(p, st);
    } else {
      fluid_gb300::Solver s(0);
      s.configure({p}, {static_cast<std::size_t>(n)});
      s.upload(st);
      s.step(steps);
      s.download(st);
    }
  } catch (const fluid_gb300::Error& e) {
    std::fprintf(stderr, "%s\n", e.what());
    return 5;
  }
  FILE* out = std::fopen(argv[2], "wb");
  for (auto* a : arr) std::fwrite(a->data(), sizeof(float), static_cast<std::size_t>(n), out);
  std::fwrite(&st.time, sizeof(float), 1, out);
  std::fclose(out);
  return 0;
}
