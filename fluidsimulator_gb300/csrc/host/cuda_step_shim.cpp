// Drop-in for the reference's CUDA backend: a maintainer adds this file to
// the reference tree in place of cuda/src/cuda_stub.cu (CMakeLists.txt:56-74,
// target fluid_cuda) and links libfluid_gb300.so. It defines the three
// functions of cuda/include/fluid/cuda.h:7-9 on top of the C ABI, so
// app/src/main.cpp (:171-184 device check, :250-251 per-step call) runs the
// GB300 step unchanged. Includes the reference's own headers.
//
// Failure behaviour (a stated difference from the reference, whose
// cuda_step checks no CUDA error and carries on): a step that fails -- the
// library's status is not FLUID_OK, for example non-finite input positions
// -- throws std::runtime_error("cuda_step: <status>") and leaves `state`
// unchanged. The reference's application calls cuda_step outside any try
// block (app/src/main.cpp:251), so there the exception ends the run through
// std::terminate; GCC's default terminate handler prints the exception's
// what() string to stderr before aborting. A failed step therefore stops the
// simulation loudly instead of writing frames of an unadvanced or corrupt
// state. A caller that wants to continue catches the exception.

#include <stdexcept>
#include <string>

#include "fluid/cuda.h"
#include "fluid_gb300.h"

namespace fluid {

int cuda_version() { return fluid_gb300_version(); }

bool cuda_device_available(int* count, const char** error) {
  return fluid_gb300_device_available(count, error) != 0;
}

void cuda_step(const Params& params, State& state) {
  fluid_params p;
  fluid_params_default(&p);
  p.dt = params.dt;
  p.density = params.density;
  p.particle_mass = params.particle_mass;
  p.h = params.h;
  p.particle_radius = params.particle_radius;
  p.epsilon = params.epsilon;
  p.solver_iterations = params.solver_iterations;
  p.neighbor_reserve_factor = params.neighbor_reserve_factor;
  p.use_uniform_grid = params.use_uniform_grid ? 1 : 0;
  p.enable_scorr = params.enable_scorr ? 1 : 0;
  p.enable_xsph = params.enable_xsph ? 1 : 0;
  p.enable_vorticity = params.enable_vorticity ? 1 : 0;
  p.scorr_k = params.scorr_k;
  p.scorr_n = params.scorr_n;
  p.scorr_dq_coeff = params.scorr_dq_coeff;
  p.visc_c = params.visc_c;
  p.plane_restitution = params.plane_restitution;
  p.plane_friction = params.plane_friction;
  p.vort_epsilon = params.vort_epsilon;
  p.vort_norm_eps = params.vort_norm_eps;
  p.external_force[0] = params.external_forces.x;
  p.external_force[1] = params.external_forces.y;
  p.external_force[2] = params.external_forces.z;
  if (params.planes.size() > FLUID_MAX_PLANES) throw std::runtime_error("cuda_step: too many planes");
  p.plane_count = static_cast<int32_t>(params.planes.size());
  for (std::size_t q = 0; q < params.planes.size(); ++q) {
    p.plane_nx[q] = params.planes.nx[q];
    p.plane_ny[q] = params.planes.ny[q];
    p.plane_nz[q] = params.planes.nz[q];
    p.plane_d[q] = params.planes.d[q];
  }
  float t = state.time;
  const int rc = fluid_gb300_cuda_step(&p, static_cast<int64_t>(state.size()), state.pos_x.data(),
                                       state.pos_y.data(), state.pos_z.data(), state.vel_x.data(),
                                       state.vel_y.data(), state.vel_z.data(), &t);
  if (rc != FLUID_OK) throw std::runtime_error(std::string("cuda_step: ") + fluid_status_string(rc));
  state.time = t;
}

}  // namespace fluid
