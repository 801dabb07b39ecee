// C++ host interface of the GB300 PBF step, mirroring the reference's backend
// API (core/include/fluid/core.h:11-135 and cuda/include/fluid/cuda.h:7-9 of
// CTKnight/FluidSimulator): the same type names, field names, defaults and
// call shapes, implemented over the C ABI in include/fluid_gb300.h. Code
// written against fluid::Params / fluid::State / fluid::cuda_step compiles
// against this namespace with the namespace swapped.
//
// Difference from the reference: cuda_step reports failures by throwing
// fluid_gb300::Error (the reference's cuda_step returns void and never checks
// CUDA errors, cuda/src/cuda_stub.cu:764-1099).
#pragma once

#include <cmath>
#include <cstddef>
#include <stdexcept>
#include <string>
#include <vector>

#include "fluid_gb300.h"

namespace fluid_gb300 {

class Error : public std::runtime_error {
 public:
  Error(int status, const std::string& what) : std::runtime_error(what), status_(status) {}
  int status() const { return status_; }

 private:
  int status_;
};

// Same fields and defaults as fluid::Params (core/include/fluid/core.h:11-79).
struct Params {
  float dt = 1.0f / 60.0f;
  enum class Backend { Cpu, Cuda };
  Backend backend = Backend::Cpu;
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
    void resize(std::size_t n) {
      nx.resize(n);
      ny.resize(n);
      nz.resize(n);
      d.resize(n);
    }
    void clear() {
      nx.clear();
      ny.clear();
      nz.clear();
      d.clear();
    }
    void add(float a, float b, float c, float dd) {
      nx.push_back(a);
      ny.push_back(b);
      nz.push_back(c);
      d.push_back(dd);
    }
    // Unit normal, d unchanged (core.h:69-77).
    void add_normalized(float a, float b, float c, float dd) {
      const float len_sq = a * a + b * b + c * c;
      if (len_sq > 0.0f) {
        const float inv = 1.0f / std::sqrt(len_sq);
        add(a * inv, b * inv, c * inv, dd);
      } else {
        add(a, b, c, dd);
      }
    }
  } planes;

  // Extension: each plane's own friction, in plane order. Empty (the
  // default) applies plane_friction to every plane, as the reference does.
  std::vector<float> plane_friction_each;

  // The C-ABI form (throws Error if there are more than FLUID_MAX_PLANES
  // planes, or if plane_friction_each is neither empty nor one per plane).
  fluid_params to_c() const;
};

// SoA particle state in caller order plus time (core.h:121-132).
struct State {
  std::vector<float> pos_x, pos_y, pos_z;
  std::vector<float> vel_x, vel_y, vel_z;
  float time = 0.0f;
  std::size_t size() const { return pos_x.size(); }
};

State make_state(std::size_t particle_count);

// cuda/include/fluid/cuda.h:7-9.
int cuda_version();
bool cuda_device_available(int* count, const char** error);
void cuda_step(const Params& params, State& state);

// Lattice block and box planes (core/src/init.cpp:72-117), for harnesses.
void init_block(const Params& params, State& state, std::size_t nx, std::size_t ny, std::size_t nz,
                float origin_x, float origin_y, float origin_z, float spacing);
void init_planes(Params& params, float box_x, float box_y, float box_z);

// Device-resident solver for one or more scenes (no reference counterpart).
class Solver {
 public:
  explicit Solver(int device = 0);
  ~Solver();
  Solver(const Solver&) = delete;
  Solver& operator=(const Solver&) = delete;

  void configure(const std::vector<Params>& scenes, const std::vector<std::size_t>& counts);
  void upload(const State& all_scenes);
  void download(State& all_scenes);
  void step(int nsteps = 1);
  float time(int scene = 0);
  fluid_stats stats();
  fluid_solver* handle() { return h_; }

 private:
  void check(int status, const char* what);
  fluid_solver* h_ = nullptr;
  std::size_t n_ = 0;
};

}  // namespace fluid_gb300
