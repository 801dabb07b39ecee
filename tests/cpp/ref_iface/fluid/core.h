// Stand-in for the reference's core/include/fluid/core.h:11-132, reduced to
// the members the drop-in shim (fluidsimulator_gb300/csrc/host/cuda_step_shim.cpp)
// reads and writes, with the reference's names, types and defaults. It lets
// the shim compile and run where the reference tree is absent (the GPU host);
// where the tree exists, tests/test_host_cpp.py also links the shim into the
// reference's own application against the real header.
#pragma once

#include <cstddef>
#include <vector>

namespace fluid {

struct Params {
  float dt = 1.0f / 60.0f;
  float density = 6000.0f;
  float particle_mass = 0.0f;
  float h = 0.0f;
  float particle_radius = 0.01f;
  float epsilon = 600.0f;
  int solver_iterations = 4;
  float neighbor_reserve_factor = 1.5f;
  bool use_uniform_grid = true;
  bool enable_scorr = false;
  bool enable_xsph = false;
  bool enable_vorticity = false;
  float scorr_k = 0.00005f;
  int scorr_n = 4;
  float scorr_dq_coeff = 0.3f;
  float visc_c = 0.0002f;
  float plane_restitution = 0.0f;
  float plane_friction = 0.0f;
  float vort_epsilon = 0.5f;
  float vort_norm_eps = 1e-6f;
  struct Vec3 {
    float x = 0.0f;
    float y = -9.8f;
    float z = 0.0f;
  } external_forces;
  struct PlaneSoA {
    std::vector<float> nx, ny, nz, d;
    std::size_t size() const { return nx.size(); }
    void add(float a, float b, float c, float e) {
      nx.push_back(a);
      ny.push_back(b);
      nz.push_back(c);
      d.push_back(e);
    }
  } planes;
};

struct State {
  std::vector<float> pos_x, pos_y, pos_z, vel_x, vel_y, vel_z;
  float time = 0.0f;
  std::size_t size() const { return pos_x.size(); }
};

}  // namespace fluid
