// ORACLE PIN — test infrastructure, not product code.
//
// C entry points over the reference's own CPU solver, compiled from the
// reference sources where they lie (core/src/core.cpp, core/src/init.cpp of
// CTKnight/FluidSimulator) by oracle/Makefile into oracle/_ref/. The tests use
// it to pin the oracle restatement (oracle/pbf_oracle.cpp) bit for bit and
// tests/golden/make_golden.py uses it to write the golden fixtures. It needs
// the reference tree at build time, so it exists only where that tree does.

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <string>

#include "fluid/core.h"
#include "fluid/init.h"
#include "fluid_gb300.h"

namespace {

fluid::Params to_ref(const fluid_params& p) {
  fluid::Params r;
  r.dt = p.dt;
  r.density = p.density;
  r.particle_mass = p.particle_mass;
  r.h = p.h;
  r.particle_radius = p.particle_radius;
  r.epsilon = p.epsilon;
  r.solver_iterations = p.solver_iterations;
  r.neighbor_reserve_factor = p.neighbor_reserve_factor;
  r.use_uniform_grid = p.use_uniform_grid != 0;
  r.enable_scorr = p.enable_scorr != 0;
  r.enable_xsph = p.enable_xsph != 0;
  r.enable_vorticity = p.enable_vorticity != 0;
  r.scorr_k = p.scorr_k;
  r.scorr_n = p.scorr_n;
  r.scorr_dq_coeff = p.scorr_dq_coeff;
  r.visc_c = p.visc_c;
  r.plane_restitution = p.plane_restitution;
  r.plane_friction = p.plane_friction;
  r.vort_epsilon = p.vort_epsilon;
  r.vort_norm_eps = p.vort_norm_eps;
  r.external_forces.x = p.external_force[0];
  r.external_forces.y = p.external_force[1];
  r.external_forces.z = p.external_force[2];
  r.planes.clear();
  for (int q = 0; q < p.plane_count; ++q) {
    r.planes.add(p.plane_nx[q], p.plane_ny[q], p.plane_nz[q], p.plane_d[q]);
  }
  return r;
}

void from_ref(const fluid::Params& r, fluid_params* p) {
  p->dt = r.dt;
  p->density = r.density;
  p->particle_mass = r.particle_mass;
  p->h = r.h;
  p->particle_radius = r.particle_radius;
  p->epsilon = r.epsilon;
  p->solver_iterations = r.solver_iterations;
  p->neighbor_reserve_factor = r.neighbor_reserve_factor;
  p->use_uniform_grid = r.use_uniform_grid;
  p->enable_scorr = r.enable_scorr;
  p->enable_xsph = r.enable_xsph;
  p->enable_vorticity = r.enable_vorticity;
  p->scorr_k = r.scorr_k;
  p->scorr_n = r.scorr_n;
  p->scorr_dq_coeff = r.scorr_dq_coeff;
  p->visc_c = r.visc_c;
  p->plane_restitution = r.plane_restitution;
  p->plane_friction = r.plane_friction;
  p->vort_epsilon = r.vort_epsilon;
  p->vort_norm_eps = r.vort_norm_eps;
  p->external_force[0] = r.external_forces.x;
  p->external_force[1] = r.external_forces.y;
  p->external_force[2] = r.external_forces.z;
  const int n = static_cast<int>(std::min<std::size_t>(r.planes.size(), FLUID_MAX_PLANES));
  p->plane_count = n;
  for (int q = 0; q < n; ++q) {
    p->plane_nx[q] = r.planes.nx[q];
    p->plane_ny[q] = r.planes.ny[q];
    p->plane_nz[q] = r.planes.nz[q];
    p->plane_d[q] = r.planes.d[q];
  }
}

}  // namespace

extern "C" {

typedef struct ref_dump {
  int32_t* cell_keys;
  int32_t* sorted_order;
  int32_t* neighbor_counts;
  float* rho;
  float* lambda;
} ref_dump;

void* ref_create(void) { return new fluid::State(fluid::make_state(0)); }
void ref_destroy(void* st) { delete static_cast<fluid::State*>(st); }

// Defaults of a freshly constructed fluid::Params, for the header-mirror test.
void ref_default_params(fluid_params* out) {
  std::memset(out, 0, sizeof(*out));
  from_ref(fluid::Params{}, out);
}

// Runs nsteps of fluid::step on the handle's State (its CpuScratch persists).
int ref_run(void* handle, const fluid_params* p, int64_t count, float* px,
            float* py, float* pz, float* vx, float* vy, float* vz, float* time,
            int32_t nsteps, const ref_dump* dump, int64_t* pairs,
            int32_t* nmax, double* dens_mean, double* dens_max) {
  // fluid::Params has one friction for all planes; a per-plane scene has no
  // reference run to pin against.
  if (p->plane_friction_per_plane) return 1;
  auto& st = *static_cast<fluid::State*>(handle);
  const fluid::Params params = to_ref(*p);
  const std::size_t n = static_cast<std::size_t>(count);
  st.pos_x.assign(px, px + n);
  st.pos_y.assign(py, py + n);
  st.pos_z.assign(pz, pz + n);
  st.vel_x.assign(vx, vx + n);
  st.vel_y.assign(vy, vy + n);
  st.vel_z.assign(vz, vz + n);
  st.time = *time;
  for (int s = 0; s < nsteps; ++s) {
    fluid::step(params, st);
    const auto& ps = st.cpu.neighbor_prefix_sum;
    if (pairs) pairs[s] = n ? static_cast<int64_t>(st.cpu.neighbor_indices.size()) : 0;
    if (nmax) {
      int32_t m = 0;
      for (std::size_t i = 0; i < n; ++i) {
        m = std::max<int32_t>(m, ps[i] - (i ? ps[i - 1] : 0));
      }
      nmax[s] = m;
    }
    if (dens_mean || dens_max) {
      double sum = 0.0, mx = -1e300;
      for (std::size_t i = 0; i < n; ++i) {
        const double e = double(st.cpu.rho[i]) / double(params.density) - 1.0;
        sum += e;
        mx = std::max(mx, e);
      }
      if (dens_mean) dens_mean[s] = n ? sum / double(n) : 0.0;
      if (dens_max) dens_max[s] = n ? mx : 0.0;
    }
  }
  std::copy(st.pos_x.begin(), st.pos_x.end(), px);
  std::copy(st.pos_y.begin(), st.pos_y.end(), py);
  std::copy(st.pos_z.begin(), st.pos_z.end(), pz);
  std::copy(st.vel_x.begin(), st.vel_x.end(), vx);
  std::copy(st.vel_y.begin(), st.vel_y.end(), vy);
  std::copy(st.vel_z.begin(), st.vel_z.end(), vz);
  *time = st.time;
  if (dump && n) {
    const auto& cpu = st.cpu;
    for (std::size_t k = 0; k < n; ++k) {
      const auto& e = cpu.grid_entries[k];
      if (dump->cell_keys) {
        dump->cell_keys[3 * e.particle + 0] = e.key.x;
        dump->cell_keys[3 * e.particle + 1] = e.key.y;
        dump->cell_keys[3 * e.particle + 2] = e.key.z;
      }
      if (dump->sorted_order) dump->sorted_order[k] = e.particle;
    }
    for (std::size_t i = 0; i < n; ++i) {
      if (dump->neighbor_counts)
        dump->neighbor_counts[i] = cpu.neighbor_prefix_sum[i] - (i ? cpu.neighbor_prefix_sum[i - 1] : 0);
      if (dump->rho) dump->rho[i] = cpu.rho[i];
      if (dump->lambda) dump->lambda[i] = cpu.lambda[i];
    }
  }
  return 0;
}

// fluid::init_block (core/src/init.cpp:72-107) into caller arrays of nx*ny*nz.
int ref_init_block(const fluid_params* p, int64_t nx, int64_t ny, int64_t nz,
                   float ox, float oy, float oz, float spacing, float* px,
                   float* py, float* pz) {
  fluid::State st = fluid::make_state(0);
  fluid::init_block(to_ref(*p), st, nx, ny, nz, ox, oy, oz, spacing);
  std::copy(st.pos_x.begin(), st.pos_x.end(), px);
  std::copy(st.pos_y.begin(), st.pos_y.end(), py);
  std::copy(st.pos_z.begin(), st.pos_z.end(), pz);
  return 0;
}

// fluid::init_planes (core/src/init.cpp:109-117) into *p.
int ref_init_planes(fluid_params* p, float bx, float by, float bz) {
  fluid::Params r = to_ref(*p);
  fluid::init_planes(r, bx, by, bz);
  from_ref(r, p);
  return 0;
}

// fluid::init_test_scene (core/src/init.cpp:119-156). Writes params and, when
// capacity suffices, the particles; *count receives the particle count.
int ref_init_test_scene(fluid_params* p, int64_t capacity, float* px, float* py,
                        float* pz, int64_t* count) {
  fluid::Params r = to_ref(*p);
  fluid::State st = fluid::make_state(0);
  fluid::init_test_scene(r, st);
  from_ref(r, p);
  *count = static_cast<int64_t>(st.size());
  if (static_cast<int64_t>(st.size()) <= capacity) {
    std::copy(st.pos_x.begin(), st.pos_x.end(), px);
    std::copy(st.pos_y.begin(), st.pos_y.end(), py);
    std::copy(st.pos_z.begin(), st.pos_z.end(), pz);
  }
  return 0;
}

// fluid::init_scene_from_json (core/src/init.cpp:158-418). Returns 0 on
// success, 1 on a loader error (message copied to err), 2 if capacity is short.
int ref_load_scene(const char* path, fluid_params* p, int64_t capacity,
                   float* px, float* py, float* pz, float* vx, float* vy,
                   float* vz, int64_t* count, char* err, int64_t err_len) {
  fluid::Params r;
  fluid::State st = fluid::make_state(0);
  std::string error;
  if (!fluid::init_scene_from_json(path, r, st, &error)) {
    if (err && err_len > 0) {
      std::strncpy(err, error.c_str(), static_cast<std::size_t>(err_len - 1));
      err[err_len - 1] = 0;
    }
    return 1;
  }
  from_ref(r, p);
  *count = static_cast<int64_t>(st.size());
  if (static_cast<int64_t>(st.size()) > capacity) return 2;
  std::copy(st.pos_x.begin(), st.pos_x.end(), px);
  std::copy(st.pos_y.begin(), st.pos_y.end(), py);
  std::copy(st.pos_z.begin(), st.pos_z.end(), pz);
  std::copy(st.vel_x.begin(), st.vel_x.end(), vx);
  std::copy(st.vel_y.begin(), st.vel_y.end(), vy);
  std::copy(st.vel_z.begin(), st.vel_z.end(), vz);
  return 0;
}

}  // extern "C"
