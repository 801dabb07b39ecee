// C++ host interface over the C ABI (see fluid_gb300.hpp).

#include "fluid_gb300.hpp"

#include <cstring>

namespace fluid_gb300 {

namespace {

void throw_status(int status, const std::string& what) {
  throw Error(status, what + ": " + fluid_status_string(status));
}

}  // namespace

fluid_params Params::to_c() const {
  fluid_params p;
  std::memset(&p, 0, sizeof(p));
  p.dt = dt;
  p.density = density;
  p.particle_mass = particle_mass;
  p.h = h;
  p.particle_radius = particle_radius;
  p.epsilon = epsilon;
  p.solver_iterations = solver_iterations;
  p.neighbor_reserve_factor = neighbor_reserve_factor;
  p.use_uniform_grid = use_uniform_grid ? 1 : 0;
  p.enable_scorr = enable_scorr ? 1 : 0;
  p.enable_xsph = enable_xsph ? 1 : 0;
  p.enable_vorticity = enable_vorticity ? 1 : 0;
  p.scorr_k = scorr_k;
  p.scorr_n = scorr_n;
  p.scorr_dq_coeff = scorr_dq_coeff;
  p.visc_c = visc_c;
  p.plane_restitution = plane_restitution;
  p.plane_friction = plane_friction;
  p.vort_epsilon = vort_epsilon;
  p.vort_norm_eps = vort_norm_eps;
  p.external_force[0] = external_forces.x;
  p.external_force[1] = external_forces.y;
  p.external_force[2] = external_forces.z;
  if (planes.size() > FLUID_MAX_PLANES) throw_status(FLUID_ERR_INVALID_ARGUMENT, "too many planes");
  p.plane_count = static_cast<int32_t>(planes.size());
  for (std::size_t q = 0; q < planes.size(); ++q) {
    p.plane_nx[q] = planes.nx[q];
    p.plane_ny[q] = planes.ny[q];
    p.plane_nz[q] = planes.nz[q];
    p.plane_d[q] = planes.d[q];
  }
  if (!plane_friction_each.empty()) {
    if (plane_friction_each.size() != planes.size())
      throw_status(FLUID_ERR_INVALID_ARGUMENT, "plane_friction_each needs one value per plane");
    p.plane_friction_per_plane = 1;
    for (std::size_t q = 0; q < planes.size(); ++q) p.plane_friction_each[q] = plane_friction_each[q];
  }
  return p;
}

State make_state(std::size_t n) {
  State s;
  s.pos_x.assign(n, 0.0f);
  s.pos_y.assign(n, 0.0f);
  s.pos_z.assign(n, 0.0f);
  s.vel_x.assign(n, 0.0f);
  s.vel_y.assign(n, 0.0f);
  s.vel_z.assign(n, 0.0f);
  return s;
}

int cuda_version() { return fluid_gb300_version(); }

bool cuda_device_available(int* count, const char** error) {
  return fluid_gb300_device_available(count, error) != 0;
}

void cuda_step(const Params& params, State& state) {
  const fluid_params p = params.to_c();
  float t = state.time;
  const int rc = fluid_gb300_cuda_step(&p, static_cast<int64_t>(state.size()), state.pos_x.data(),
                                       state.pos_y.data(), state.pos_z.data(), state.vel_x.data(),
                                       state.vel_y.data(), state.vel_z.data(), &t);
  if (rc) throw_status(rc, "cuda_step");
  state.time = t;
}

void init_block(const Params&, State& state, std::size_t nx, std::size_t ny, std::size_t nz, float ox, float oy,
                float oz, float spacing) {
  state = make_state(nx * ny * nz);
  std::size_t k = 0;
  for (std::size_t z = 0; z < nz; ++z)
    for (std::size_t y = 0; y < ny; ++y)
      for (std::size_t x = 0; x < nx; ++x, ++k) {
        state.pos_x[k] = ox + static_cast<float>(x) * spacing;
        state.pos_y[k] = oy + static_cast<float>(y) * spacing;
        state.pos_z[k] = oz + static_cast<float>(z) * spacing;
      }
}

void init_planes(Params& params, float bx, float by, float bz) {
  params.planes.clear();
  params.planes.add_normalized(1.0f, 0.0f, 0.0f, 0.0f);
  params.planes.add_normalized(-1.0f, 0.0f, 0.0f, -bx);
  params.planes.add_normalized(0.0f, 1.0f, 0.0f, 0.0f);
  params.planes.add_normalized(0.0f, -1.0f, 0.0f, -by);
  params.planes.add_normalized(0.0f, 0.0f, 1.0f, 0.0f);
  params.planes.add_normalized(0.0f, 0.0f, -1.0f, -bz);
}

Solver::Solver(int device) {
  const int rc = fluid_solver_create(&h_, device);
  if (rc) throw_status(rc, "fluid_solver_create");
}

Solver::~Solver() { fluid_solver_destroy(h_); }

void Solver::check(int status, const char* what) {
  if (status) throw Error(status, std::string(what) + ": " + fluid_solver_last_error(h_));
}

void Solver::configure(const std::vector<Params>& scenes, const std::vector<std::size_t>& counts) {
  std::vector<fluid_params> ps;
  std::vector<int64_t> cs;
  n_ = 0;
  for (const auto& s : scenes) ps.push_back(s.to_c());
  for (auto c : counts) {
    cs.push_back(static_cast<int64_t>(c));
    n_ += c;
  }
  check(fluid_solver_configure(h_, static_cast<int32_t>(ps.size()), ps.data(), cs.data()), "configure");
}

void Solver::upload(const State& s) {
  check(fluid_solver_upload(h_, s.pos_x.data(), s.pos_y.data(), s.pos_z.data(), s.vel_x.data(), s.vel_y.data(),
                            s.vel_z.data(), FLUID_MEMORY_HOST),
        "upload");
}

void Solver::download(State& s) {
  if (s.size() != n_) s = make_state(n_);
  check(fluid_solver_download(h_, s.pos_x.data(), s.pos_y.data(), s.pos_z.data(), s.vel_x.data(), s.vel_y.data(),
                              s.vel_z.data(), FLUID_MEMORY_HOST),
        "download");
  check(fluid_solver_get_time(h_, 0, &s.time), "time");
}

void Solver::step(int nsteps) { check(fluid_solver_step(h_, nsteps), "step"); }

float Solver::time(int scene) {
  float t = 0.0f;
  check(fluid_solver_get_time(h_, scene, &t), "time");
  return t;
}

fluid_stats Solver::stats() {
  fluid_stats st;
  check(fluid_solver_get_stats(h_, &st), "stats");
  return st;
}

}  // namespace fluid_gb300
