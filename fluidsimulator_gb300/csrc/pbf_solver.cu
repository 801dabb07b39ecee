// Host runtime of the GB300 PBF timestep and the C ABI of include/fluid_gb300.h.
//
// A Solver owns the device-resident state of one or more independent scenes
// (all scenes run in the same launches; each particle carries its scene id),
// the step scratch, capacity management for the neighbour lists and the cell
// table, CUDA-graph capture of the step, and optional per-launch timing.

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "fluid_gb300.h"
#include "pbf_adjoint.h"
#include "pbf_common.cuh"
#include "pbf_launch.h"

namespace fgb {
namespace {

constexpr float kPi = 3.14159265358979323846f;  // core/src/core.cpp:10

// Owning device buffer; move-only so containers never double-free.
template <typename T>
struct DBuf {
  T* p = nullptr;
  size_t n = 0;
  DBuf() = default;
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  DBuf(DBuf&& o) noexcept : p(o.p), n(o.n) {
    o.p = nullptr;
    o.n = 0;
  }
  DBuf& operator=(DBuf&& o) noexcept {
    if (this != &o) {
      release();
      p = o.p;
      n = o.n;
      o.p = nullptr;
      o.n = 0;
    }
    return *this;
  }
  cudaError_t alloc(size_t count) {
    release();
    if (count == 0) return cudaSuccess;
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&p), count * sizeof(T));
    if (e != cudaSuccess) {
      p = nullptr;
      return e;
    }
    n = count;
    return cudaSuccess;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  ~DBuf() { release(); }
};

// poly6_kernel (core/src/core.cpp:35-46), host float arithmetic.
float poly6_host(float r2, float h) {
  const float h2 = h * h;
  if (r2 > h2) return 0.0f;
  const float diff = h2 - r2;
  const float diff3 = diff * diff * diff;
  const float h4 = h2 * h2;
  const float h9 = h4 * h4 * h;
  const float coeff = 315.0f / (64.0f * kPi * h9);
  return coeff * diff3;
}

// Per-scene constants, each from the same float expression the reference
// evaluates (core/src/core.cpp:138-148, :270-274, :35-57).
SceneConst make_scene_const(const fluid_params& p, int first, int count) {
  SceneConst c;
  std::memset(&c, 0, sizeof(c));
  const float h = p.h;
  c.h = h;
  c.inv_h = 1.0f / h;
  c.h2 = h * h;
  const float min_r = 0.01f * h;
  c.min_r2 = min_r * min_r;
  {
    const float h2 = h * h;
    const float h4 = h2 * h2;
    const float h9 = h4 * h4 * h;
    c.poly6_c = 315.0f / (64.0f * kPi * h9);
    c.w0 = poly6_host(0.0f, h);
    const float h6 = h2 * h2 * h2;
    c.spiky_c = -45.0f / (kPi * h6);
  }
  c.mass = p.particle_mass;
  c.density = p.density;
  c.inv_density = 1.0f / p.density;
  c.grad_scale = p.particle_mass * c.inv_density;
  c.epsilon = p.epsilon;
  const bool scorr = p.enable_scorr && p.scorr_k != 0.0f;
  const float dq_coeff = (p.scorr_dq_coeff > 0.0f) ? p.scorr_dq_coeff : 0.3f;
  const float dq = dq_coeff * h;
  const float wdq = scorr ? poly6_host(dq * dq, h) : 0.0f;
  c.scorr_inv_wdq = (wdq > 1e-12f) ? (1.0f / wdq) : 0.0f;
  c.scorr_on = (scorr && c.scorr_inv_wdq > 0.0f) ? 1 : 0;
  c.scorr_neg_k = -p.scorr_k;
  c.scorr_n = p.scorr_n;
  c.dt = p.dt;
  c.gdt_x = p.external_force[0] * p.dt;
  c.gdt_y = p.external_force[1] * p.dt;
  c.gdt_z = p.external_force[2] * p.dt;
  c.visc_c = p.visc_c;
  c.xsph_on = (p.enable_xsph && p.visc_c != 0.0f) ? 1 : 0;
  c.vort_eps = p.vort_epsilon;
  c.vort_norm_eps = p.vort_norm_eps;
  c.vort_on = (p.enable_vorticity && p.vort_epsilon != 0.0f) ? 1 : 0;
  // core.cpp:573-612 with one friction for every plane, or each plane's own
  // when plane_friction_per_plane is set.
  c.rest_neg_e = -p.plane_restitution;
  bool friction = false;
  for (int q = 0; q < p.plane_count; ++q) {
    const float mu = p.plane_friction_per_plane ? p.plane_friction_each[q] : p.plane_friction;
    c.rest_scale[q] = 1.0f - mu;
    friction |= mu > 0.0f;
  }
  c.rest_on = ((p.plane_restitution > 0.0f || friction) && p.plane_count > 0) ? 1 : 0;
  c.plane_count = p.plane_count;
  c.iterations = p.solver_iterations;
  c.all_pairs = p.use_uniform_grid ? 0 : 1;
  c.first_slot = first;
  c.neg_zero = -0.0f;
  c.exact_sqrt = rn_sqrt_covers(c.min_r2, c.h2) ? 0 : 1;
  c.count = count;
  for (int q = 0; q < p.plane_count; ++q) {
    c.planes[q] = make_float4(p.plane_nx[q], p.plane_ny[q], p.plane_nz[q], p.plane_d[q]);
  }
  return c;
}

int validate_params(const fluid_params& p, std::string& why) {
  auto bad = [&](const char* m) {
    why = m;
    return static_cast<int>(FLUID_ERR_INVALID_ARGUMENT);
  };
  if (!(p.dt > 0.0f) || !std::isfinite(p.dt)) return bad("dt must be finite and > 0");
  if (!(p.h > 0.0f) || !std::isfinite(p.h)) return bad("h must be finite and > 0");
  if (!(p.density > 0.0f) || !std::isfinite(p.density)) return bad("density must be finite and > 0");
  if (!std::isfinite(p.particle_mass)) return bad("particle_mass must be finite");
  if (p.solver_iterations < 0) return bad("solver_iterations must be >= 0");
  if (p.plane_count < 0 || p.plane_count > FLUID_MAX_PLANES) return bad("plane_count out of range");
  return FLUID_OK;
}

long long round_up(long long v, long long m) { return (v + m - 1) / m * m; }

int bits_for(long long cap) {
  if (cap <= 1) return 0;
  int b = 0;
  unsigned long long v = static_cast<unsigned long long>(cap - 1);
  while (v) {
    ++b;
    v >>= 1;
  }
  return b;
}

}  // namespace

// Device address of a page-locked host buffer of `bytes` bytes mapped for
// `device` (pinned by cudaHostAlloc / cudaMallocHost or registered with
// cudaHostRegister), or nullptr for any other memory. Both the first and the
// last byte must lie in the same mapping (a registered range shorter than
// the array would otherwise let the kernels run past it over the host link).
// The upload and download kernels read and write such buffers in place,
// without staging copies; any other memory keeps the copy path.
const void* mapped_host(const void* p, size_t bytes, int device) {
  auto lookup = [device](const void* q) -> const char* {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, q) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    if (at.type != cudaMemoryTypeHost || !at.devicePointer || at.device != device) return nullptr;
    return static_cast<const char*>(at.devicePointer);
  };
  const char* first = lookup(p);
  if (!first || bytes == 0) return first;
  const char* last_host = static_cast<const char*>(p) + (bytes - 1);
  const char* last = lookup(last_host);
  if (!last || last != first + (bytes - 1)) return nullptr;
  return first;
}

class Solver {
 public:
  explicit Solver(int device) : device_(device) {}
  ~Solver() {
    if (device_ >= 0) cudaSetDevice(device_);
    destroy_graphs();
    destroy_events();
    for (int k = 0; k < 2; ++k) {
      if (frame_busy_[k]) cudaEventSynchronize(frame_done_[k]);
      if (frame_gather_[k]) cudaEventDestroy(frame_gather_[k]);
      if (frame_done_[k]) cudaEventDestroy(frame_done_[k]);
    }
    if (copy_stream_) cudaStreamDestroy(copy_stream_);
    if (status_host_) cudaFreeHost(status_host_);
    if (split_.committed) cudaEventDestroy(split_.committed);
    if (split_.positions_done) cudaEventDestroy(split_.positions_done);
    if (aux_) cudaStreamDestroy(aux_);
    if (targets_host_) cudaFreeHost(targets_host_);
    if (own_) cudaStreamDestroy(own_);
  }

  int init() {
    if (cudaSetDevice(device_) != cudaSuccess) return cuda_fail("cudaSetDevice");
    if (cudaStreamCreateWithFlags(&own_, cudaStreamNonBlocking) != cudaSuccess) return cuda_fail("stream");
    stream_ = own_;
    if (cudaMallocHost(reinterpret_cast<void**>(&status_host_), sizeof(DevStatus)) != cudaSuccess)
      return cuda_fail("cudaMallocHost");
    if (status_.alloc(1) != cudaSuccess) return cuda_fail("cudaMalloc status");
    cudaMemset(status_.p, 0, sizeof(DevStatus));
    return FLUID_OK;
  }

  int set_stream(void* s) {
    int rc = synchronize();
    if (rc) return rc;
    stream_ = s ? static_cast<cudaStream_t>(s) : own_;
    invalidate_graphs();
    return FLUID_OK;
  }

  int configure(int scenes, const fluid_params* params, const int64_t* counts) {
    if (scenes < 1 || !params || !counts) return fail(FLUID_ERR_INVALID_ARGUMENT, "need >= 1 scene");
    long long total = 0;
    for (int s = 0; s < scenes; ++s) {
      std::string why;
      int rc = validate_params(params[s], why);
      if (rc) return fail(rc, "scene " + std::to_string(s) + ": " + why);
      if (counts[s] < 0) return fail(FLUID_ERR_INVALID_ARGUMENT, "negative particle count");
      if (params[s].solver_iterations != params[0].solver_iterations)
        return fail(FLUID_ERR_NOT_SUPPORTED, "all scenes must share solver_iterations");
      total += counts[s];
    }
    if (total >= (1ll << 30)) return fail(FLUID_ERR_INVALID_ARGUMENT, "2^30 or more particles");
    cudaSetDevice(device_);
    int rc = synchronize_quiet();
    (void)rc;
    destroy_graphs();
    S_ = scenes;
    n_ = static_cast<int>(total);
    params_.assign(params, params + scenes);
    counts_.assign(counts, counts + scenes);
    times_.assign(scenes, 0.0f);
    steps_ = 0;
    regrows_ = 0;
    grows_ahead_ = 0;
    last_list_ints_ = 0;
    parity_ = 0;
    pending_ = 0;
    uploaded_ = false;
    build_scene_consts();
    plan_ = StepPlan();
    plan_.size_for(n_);
    checkpoints_.clear();
    tapes_.clear();
    rec_steps_ = 0;
    tail_taped_ = false;
    adj_n_ = 0;
    warps_ = (n_ + 31) / 32;
    tiles_ = std::max(1, (n_ + kRadixTile - 1) / kRadixTile);
    const size_t n = static_cast<size_t>(std::max(n_, 1));
    const size_t np = static_cast<size_t>(round_up(n, 32));
    bool ok = true;
    for (int k = 0; k < 2; ++k) {
      ok &= x_[k].alloc(np) == cudaSuccess;
      ok &= v_[k].alloc(np) == cudaSuccess;
      ok &= p_[k].alloc(np) == cudaSuccess;
      ok &= slot_[k].alloc(np) == cudaSuccess;
      ok &= rho_[k].alloc(np) == cudaSuccess;
      ok &= keys_[k].alloc(np) == cudaSuccess;
      ok &= vals_[k].alloc(np) == cudaSuccess;
    }
    ok &= v2_.alloc(np) == cudaSuccess;
    ok &= omega_.alloc(np) == cudaSuccess;
    ok &= pl_.alloc(np) == cudaSuccess;
    ok &= live_.alloc(2 * np) == cudaSuccess;
    ok &= lambda_.alloc(np) == cudaSuccess;
    ok &= cnt_.alloc(np) == cudaSuccess;
    ok &= depth_.alloc(static_cast<size_t>(warps_) + 1) == cudaSuccess;
    ok &= ovf_.alloc(static_cast<size_t>(warps_) + 1) == cudaSuccess;
    ok &= wbase_.alloc(static_cast<size_t>(warps_) + 1) == cudaSuccess;
    ok &= look_.alloc(static_cast<size_t>(tiles_) * kRadixMaxBins) == cudaSuccess;
    ok &= radix_next_.alloc(kRadixMaxPasses) == cudaSuccess;
    ok &= digit_total_.alloc(kRadixMaxPasses * kRadixMaxBins) == cudaSuccess;
    ok &= bmin_.alloc(3 * static_cast<size_t>(S_)) == cudaSuccess;
    ok &= bmax_.alloc(3 * static_cast<size_t>(S_)) == cudaSuccess;
    ok &= grid_.alloc(static_cast<size_t>(S_)) == cudaSuccess;
    ok &= sc_.alloc(static_cast<size_t>(S_)) == cudaSuccess;
    if (!ok) return fail(FLUID_ERR_OUT_OF_MEMORY, "device allocation failed");
    grid_cap_ = std::max<long long>(1 << 16, 4ll * n_);
    nbr_cap_ = 48ll * 32 * warps_;
    if (table_.alloc(static_cast<size_t>(grid_cap_)) != cudaSuccess ||
        nbr_.alloc(static_cast<size_t>(nbr_cap_)) != cudaSuccess)
      return fail(FLUID_ERR_OUT_OF_MEMORY, "device allocation failed");
    cudaMemsetAsync(table_.p, 0, table_.n * sizeof(int2), stream_);
    cudaMemsetAsync(look_.p, 0, look_.n * sizeof(unsigned long long), stream_);  // tag 0: never current
    if (cudaMemcpyAsync(sc_.p, sc_host_.data(), S_ * sizeof(SceneConst), cudaMemcpyHostToDevice, stream_) !=
        cudaSuccess)
      return cuda_fail("upload scene constants");
    if (enqueue_reset(status_.p, bmin_.p, bmax_.p, S_, stream_) != cudaSuccess) return cuda_fail("reset");
    if (cudaStreamSynchronize(stream_) != cudaSuccess) return cuda_fail("configure");
    make_plan();
    return FLUID_OK;
  }

  int set_params(const fluid_params* params) {
    if (!S_) return fail(FLUID_ERR_STATE, "configure first");
    // Unchanged parameters (the usual case of a caller stepping one scene
    // repeatedly) need no validation, upload or synchronisation.
    if (params && std::memcmp(params, params_.data(), sizeof(fluid_params) * S_) == 0) return FLUID_OK;
    for (int s = 0; s < S_; ++s) {
      std::string why;
      int rc = validate_params(params[s], why);
      if (rc) return fail(rc, why);
      if (params[s].solver_iterations != params[0].solver_iterations)
        return fail(FLUID_ERR_NOT_SUPPORTED, "all scenes must share solver_iterations");
    }
    int rc = synchronize();
    if (rc) return rc;
    params_.assign(params, params + S_);
    tail_taped_ = false;
    build_scene_consts();
    if (cudaMemcpyAsync(sc_.p, sc_host_.data(), S_ * sizeof(SceneConst), cudaMemcpyHostToDevice, stream_) !=
            cudaSuccess ||
        cudaStreamSynchronize(stream_) != cudaSuccess)
      return cuda_fail("set_params");
    StepPlan old = plan_;
    make_plan();
    if (old.iterations != plan_.iterations || old.xsph != plan_.xsph || old.vorticity != plan_.vorticity ||
        old.restitution != plan_.restitution || old.scorr_pow != plan_.scorr_pow)
      invalidate_graphs();
    return FLUID_OK;
  }

  // wait = false leaves the copies in flight on the solver's stream, for a
  // caller whose next work on that stream consumes them (the stateless step).
  // bounds: for page-locked arrays, the upload kernel also adds the
  // predicted cells to the bounding box and the next step_download_host
  // skips k_bounds (the stateless step).
  int upload(const float* px, const float* py, const float* pz, const float* vx, const float* vy,
             const float* vz, int memory, bool wait = true, bool bounds = false) {
    if (!S_) return fail(FLUID_ERR_STATE, "configure first");
    if (n_ > 0 && (!px || !py || !pz || !vx || !vy || !vz)) return fail(FLUID_ERR_INVALID_ARGUMENT, "null array");
    int rc = synchronize();
    if (rc) return rc;
    bounds_ready_ = false;
    if (n_ > 0) {
      const float* src[6] = {px, py, pz, vx, vy, vz};
      const float* dev[6];
      if (memory == FLUID_MEMORY_HOST && all_mapped(src, dev)) {
        // page-locked: the upload kernel reads the caller's arrays in place
        bounds_ready_ = bounds;
      } else if (memory == FLUID_MEMORY_HOST) {
        float* stage = reinterpret_cast<float*>(p_[0].p);  // 4n floats
        float* stage2 = reinterpret_cast<float*>(p_[1].p);
        for (int k = 0; k < 6; ++k) {
          float* dst = (k < 4 ? stage : stage2) + static_cast<size_t>(k % 4) * n_;
          if (cudaMemcpyAsync(dst, src[k], sizeof(float) * n_, cudaMemcpyHostToDevice, stream_) != cudaSuccess)
            return cuda_fail("upload copy");
          dev[k] = dst;
        }
      } else {
        for (int k = 0; k < 6; ++k) dev[k] = src[k];
      }
      if (enqueue_upload(dev[0], dev[1], dev[2], dev[3], dev[4], dev[5], x_[parity_].p, v_[parity_].p,
                         slot_[parity_].p, rho_[parity_].p, sc_.p, S_, n_, stream_,
                         bounds_ready_ ? bmin_.p : nullptr, bounds_ready_ ? bmax_.p : nullptr) != cudaSuccess)
        return cuda_fail("upload kernel");
      if (wait && cudaStreamSynchronize(stream_) != cudaSuccess) return cuda_fail("upload");
    }
    uploaded_ = true;
    last_list_ints_ = 0;  // a new state: its lists' growth starts over
    return FLUID_OK;
  }

  int download(float* px, float* py, float* pz, float* vx, float* vy, float* vz, int memory) {
    if (!uploaded_) return fail(FLUID_ERR_STATE, "no state uploaded");
    if (n_ > 0 && (!px || !py || !pz || !vx || !vy || !vz)) return fail(FLUID_ERR_INVALID_ARGUMENT, "null array");
    int rc = synchronize();
    if (rc) return rc;
    if (n_ == 0) return FLUID_OK;
    float* dst[6] = {px, py, pz, vx, vy, vz};
    float* dev[6];
    bool staged = false;
    if (memory == FLUID_MEMORY_HOST && all_mapped(dst, dev)) {
      // page-locked: the download kernel writes the caller's arrays in place
    } else if (memory == FLUID_MEMORY_HOST) {
      float* stage = reinterpret_cast<float*>(p_[0].p);
      float* stage2 = reinterpret_cast<float*>(p_[1].p);
      for (int k = 0; k < 6; ++k) dev[k] = (k < 4 ? stage : stage2) + static_cast<size_t>(k % 4) * n_;
      staged = true;
    } else {
      for (int k = 0; k < 6; ++k) dev[k] = dst[k];
    }
    if (enqueue_download(x_[parity_].p, v_[parity_].p, slot_[parity_].p, dev[0], dev[1], dev[2], dev[3], dev[4],
                         dev[5], n_, stream_) != cudaSuccess)
      return cuda_fail("download kernel");
    if (staged) {
      for (int k = 0; k < 6; ++k) {
        if (cudaMemcpyAsync(dst[k], dev[k], sizeof(float) * n_, cudaMemcpyDeviceToHost, stream_) != cudaSuccess)
          return cuda_fail("download copy");
      }
    }
    if (cudaStreamSynchronize(stream_) != cudaSuccess) return cuda_fail("download");
    return FLUID_OK;
  }

  // Device addresses of six host arrays when every one is page-locked and
  // mapped for this solver's device.
  template <typename T>
  bool all_mapped(T* const (&host)[6], T* (&dev)[6]) const {
    for (int k = 0; k < 6; ++k) {
      const void* d = mapped_host(host[k], sizeof(T) * static_cast<size_t>(n_), device_);
      if (!d) return false;
      dev[k] = static_cast<T*>(const_cast<void*>(d));
    }
    return true;
  }

  // One step whose result goes straight into the caller's page-locked host
  // arrays while the step finishes (StepDownload: positions beside the
  // velocity passes, velocities at the end), launched without the graph;
  // any other memory takes step + download.
  int step_download_host(float* px, float* py, float* pz, float* vx, float* vy, float* vz) {
    float* host[6] = {px, py, pz, vx, vy, vz};
    float* dev[6];
    if (n_ == 0 || profiling_ || !all_mapped(host, dev)) {
      int rc = step(1);
      return rc ? rc : download(px, py, pz, vx, vy, vz, FLUID_MEMORY_HOST);
    }
    if (!aux_) {
      if (cudaStreamCreateWithFlags(&aux_, cudaStreamNonBlocking) != cudaSuccess ||
          cudaEventCreateWithFlags(&split_.committed, cudaEventDisableTiming) != cudaSuccess ||
          cudaEventCreateWithFlags(&split_.positions_done, cudaEventDisableTiming) != cudaSuccess ||
          targets_.alloc(6) != cudaSuccess ||
          cudaMallocHost(reinterpret_cast<void**>(&targets_host_), 6 * sizeof(float*)) != cudaSuccess)
        return cuda_fail("download stream");
      split_.aux = aux_;
      split_.targets = targets_.p;
      int sms = 0;
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device_);
      split_.blocks = sms > 4 ? sms / 4 : 1;
    }
    int rc = synchronize();  // targets_host_ may still feed an earlier copy
    if (rc) return rc;
    for (int k = 0; k < 6; ++k) targets_host_[k] = dev[k];
    if (cudaMemcpyAsync(targets_.p, targets_host_, 6 * sizeof(float*), cudaMemcpyHostToDevice, stream_) !=
        cudaSuccess)
      return cuda_fail("download targets");
    split_on_ = true;
    rc = step(1);  // a step re-run after regrowth writes out again
    split_on_ = false;
    return rc;
  }

  int step_async(int nsteps) {
    if (!uploaded_) return fail(FLUID_ERR_STATE, "no state uploaded");
    if (nsteps < 0) return fail(FLUID_ERR_INVALID_ARGUMENT, "negative step count");
    if (n_ == 0) {
      for (int k = 0; k < nsteps; ++k) advance_times(1);
      steps_ += nsteps;
      return FLUID_OK;
    }
    for (int k = 0; k < nsteps; ++k) {
      int rc = launch_one();
      if (rc) return rc;
    }
    return FLUID_OK;
  }

  int step(int nsteps) {
    int rc = step_async(nsteps);
    if (rc) return rc;
    return synchronize();
  }

  // Waits for the enqueued steps; steps that overflowed a capacity are
  // re-run after growing it.
  int synchronize() {
    for (;;) {
      if (pending_ == 0) return FLUID_OK;
      if (cudaMemcpyAsync(status_host_, status_.p, sizeof(DevStatus), cudaMemcpyDeviceToHost, stream_) !=
          cudaSuccess)
        return cuda_fail("status read");
      if (cudaStreamSynchronize(stream_) != cudaSuccess) return cuda_fail("step");
      const DevStatus st = *status_host_;
      const int done = st.err ? st.fail_step : pending_;
      const int remaining = pending_ - done;
      // Each parity's events hold its latest step: the last two completed
      // steps are timed (every step when the caller synchronises each step).
      if (profiling_)
        for (int k = std::max(0, done - 2); k < done; ++k) accumulate_profile((parity_ + k) & 1);
      commit_steps(done);
      pending_ = 0;
      last_pairs_ = static_cast<long long>(st.pairs);
      last_max_ = st.nbr_max;
      last_cells_ = static_cast<int>(st.total_cells);
      last_npass_ = st.npass;
      if (enqueue_reset(status_.p, bmin_.p, bmax_.p, S_, stream_) != cudaSuccess) return cuda_fail("reset");
      if (!st.err) {
        adapt_stage_rows(st.nbr_max);
        return grow_ahead(st.cursor);
      }
      if (st.err != FLUID_ERR_CAPACITY) {
        cudaStreamSynchronize(stream_);
        return fail(st.err, st.err == FLUID_ERR_NONFINITE ? "non-finite predicted position"
                            : st.err == FLUID_ERR_CUDA    ? "sort look-back did not complete"
                                                          : "particle cells span too large a grid");
      }
      int rc = grow(st.need_grid, st.cursor);
      if (rc) return rc;
      ++regrows_;
      for (int k = 0; k < remaining; ++k) {
        rc = launch_one();
        if (rc) return rc;
      }
    }
  }

  int set_graphs(int on) {
    int rc = synchronize();
    if (rc) return rc;
    use_graphs_ = on != 0;
    invalidate_graphs();
    return FLUID_OK;
  }

  int set_profiling(int on) {
    int rc = synchronize();
    if (rc) return rc;
    profiling_ = on != 0;
    invalidate_graphs();
    if (profiling_) {
      for (int k = 0; k < 2; ++k) {
        if (events_[k].empty()) {
          events_[k].resize(64);
          stages_[k].assign(64, 0);
          for (auto& e : events_[k]) cudaEventCreate(&e);
        }
      }
    }
    return FLUID_OK;
  }

  // Times every tunable kernel under each (unroll, block) shape on the
  // current state and keeps the fastest shape per kernel. Trial steps are
  // discarded (the step's input stays in the current parity buffers), so the
  // state is not advanced. All shapes compute identical results.
  int autotune(int trials) {
    if (!uploaded_) return fail(FLUID_ERR_STATE, "no state uploaded");
    int rc = synchronize();
    if (rc) return rc;
    if (n_ == 0) return FLUID_OK;
    trials = std::max(1, trials);
    const int parity0 = parity_;
    const long long steps0 = steps_;
    const std::vector<float> times0 = times_;
    auto revert = [&] {
      parity_ = parity0;
      steps_ = steps0;
      times_ = times0;
    };
    rc = step(1);  // sizes the lists and the cell table for this state
    revert();
    if (rc) return rc;
    const bool prof = profiling_;
    rc = set_profiling(1);
    if (rc) return rc;
    StepPlan best = plan_;
    double best_ms[FLUID_KERNEL_COUNT];
    std::fill(std::begin(best_ms), std::end(best_ms), 1e300);
    // Each kernel's default shape (4 ahead; 128 threads for the list passes,
    // 256 for the build; the default lanes for this particle count) is timed first and another replaces the best only
    // when at least 2 % faster, so a kernel that runs alike under several
    // shapes in the tuned state keeps its default rather than a noise pick. One entry ahead is left out: with short lists (all
    // within the live-bit head of the vorticity passes) it can win by a few
    // per cent on register count, and it is ~2x slower once lists grow.
    // Then several lanes per particle (2, 4, 8) at each block size, for the
    // list passes only (the list build keeps its one-lane shape).
    const int unrolls[] = {4, 2, 8};
    const int blocks[] = {128, 256, 512};
    struct Shape {
      int u, b, g;  // b = 0, g = 0: each kernel's default block, lanes
    };
    StepPlan defaults;
    defaults.size_for(n_);
    std::vector<Shape> shapes{{4, 0, 0}};
    for (int u : unrolls)
      for (int b : blocks) shapes.push_back({u, b, 1});
    for (int g : {2, 4, 8})
      for (int b : blocks) shapes.push_back({4, b, g});
    for (const Shape& sh : shapes) {
      const int u = sh.u, b = sh.b, g = sh.g;
      {
        for (int k = 0; k < FLUID_KERNEL_COUNT; ++k) {
          if (tunable_unroll(k)) {
            plan_.unroll[k] = u;
            plan_.lanes[k] = g == 0 ? defaults.lanes[k] : g;
          }
          if (tunable_block(k))
            plan_.block[k] = b == 0 ? defaults.block[k] : (g == 1 || tunable_unroll(k) ? b : best.block[k]);
        }
        invalidate_graphs();
        kernel_times(nullptr, nullptr, 0, 1);
        for (int t = 0; t < trials; ++t) {
          rc = launch_one();
          if (!rc) rc = synchronize();
          revert();
          if (rc) {
            plan_ = best;
            set_profiling(prof);
            return rc;
          }
        }
        for (int k = 0; k < FLUID_KERNEL_COUNT; ++k) {
          if (!tunable_block(k) || stage_launches_[k] == 0) continue;
          if (k == FLUID_KERNEL_NBR_BUILD && b > 256) continue;  // launched at 256 regardless
          if (g > 1 && !tunable_unroll(k)) continue;              // not a list pass
          const double avg = stage_ms_[k] / static_cast<double>(stage_launches_[k]);
          if (avg < 0.98 * best_ms[k]) {
            best_ms[k] = avg;
            if (tunable_unroll(k)) {
              best.unroll[k] = u;
              best.lanes[k] = plan_.lanes[k];
            }
            best.block[k] = plan_.block[k];  // the block this shape launched (b = 0: the default)
          }
        }
      }
    }
    for (int k = 0; k < FLUID_KERNEL_COUNT; ++k) {
      plan_.unroll[k] = best.unroll[k];
      plan_.block[k] = best.block[k];
      plan_.lanes[k] = best.lanes[k];
    }
    // Sort digit width: the three radix stages' time per step under each.
    double best_sort = 1e300;
    int best_bits = plan_.radix_bits;
    for (int bits : {8, 9, 11}) {
      plan_.radix_bits = bits;
      make_plan();
      invalidate_graphs();
      kernel_times(nullptr, nullptr, 0, 1);
      for (int t = 0; t < trials; ++t) {
        rc = launch_one();
        if (!rc) rc = synchronize();
        revert();
        if (rc) break;
      }
      if (rc) break;
      const double ms = stage_ms_[FLUID_KERNEL_RADIX_HIST] + stage_ms_[FLUID_KERNEL_RADIX_SCAN] +
                        stage_ms_[FLUID_KERNEL_RADIX_SCATTER];
      if (ms < best_sort) {
        best_sort = ms;
        best_bits = bits;
      }
    }
    plan_.radix_bits = best_bits;
    make_plan();
    kernel_times(nullptr, nullptr, 0, 1);
    invalidate_graphs();
    const int prof_rc = set_profiling(prof);
    return rc ? rc : prof_rc;
  }

  int sort_bits() const { return plan_.radix_bits; }

  int set_sort_bits(int bits) {
    if (bits != 8 && bits != 9 && bits != 11)
      return fail(FLUID_ERR_INVALID_ARGUMENT, "sort digit width must be 8, 9 or 11");
    int rc = synchronize();
    if (rc) return rc;
    plan_.radix_bits = bits;
    make_plan();
    invalidate_graphs();
    return FLUID_OK;
  }

  // ---- Adjoint -----------------------------------------------------------

  // Vector-Jacobian product of the step the current state would take, all
  // pointers on the device (3n floats: x, y, z blocks, caller order). The
  // state, time and step count are left unchanged.
  int vjp_device(const float* gpo, const float* gvo, float* gpi, float* gvi, std::vector<double>& gc) {
    if (!uploaded_) return fail(FLUID_ERR_STATE, "no state uploaded");
    int rc = synchronize();
    if (rc) return rc;
    gc.assign(S_, 0.0);
    if (n_ == 0) return FLUID_OK;
    if ((rc = ensure_adjoint_buffers())) return rc;
    if (tapes_.empty()) tapes_.resize(1);
    tail_taped_ = false;  // tapes_[0] is overwritten below
    const int parity0 = parity_;
    const long long steps0 = steps_;
    const std::vector<float> times0 = times_;
    rc = taped_step(tapes_[0]);
    parity_ = parity0;  // the step's input is still in these buffers
    steps_ = steps0;
    times_ = times0;
    if (rc) return rc;
    return tape_adjoint(tapes_[0], gpo, gvo, gpi, gvi, gc);
  }

  int step_backward(const float* gpo, const float* gvo, float* gpi, float* gvi, float* gvisc, int memory) {
    if (!gpo || !gvo || !gpi || !gvi) return fail(FLUID_ERR_INVALID_ARGUMENT, "null cotangent");
    int rc = synchronize();
    if (rc) return rc;
    if ((rc = ensure_adjoint_buffers())) return rc;
    const size_t b = 3 * static_cast<size_t>(n_) * sizeof(float);
    float* io = a_io_.p;
    const size_t m3 = 3 * static_cast<size_t>(n_);
    const float *dpo = gpo, *dvo = gvo;
    float *dpi = gpi, *dvi = gvi;
    if (memory == FLUID_MEMORY_HOST) {
      cudaMemcpy(io, gpo, b, cudaMemcpyHostToDevice);
      cudaMemcpy(io + m3, gvo, b, cudaMemcpyHostToDevice);
      dpo = io;
      dvo = io + m3;
      dpi = io + 2 * m3;
      dvi = io + 3 * m3;
    }
    std::vector<double> gc;
    if ((rc = vjp_device(dpo, dvo, dpi, dvi, gc))) return rc;
    if (memory == FLUID_MEMORY_HOST) {
      cudaMemcpy(gpi, dpi, b, cudaMemcpyDeviceToHost);
      cudaMemcpy(gvi, dvi, b, cudaMemcpyDeviceToHost);
    }
    if (gvisc)
      for (int sc = 0; sc < S_; ++sc) gvisc[sc] = static_cast<float>(gc[sc]);
    return FLUID_OK;
  }

  // Forward nsteps from the current state keeping a snapshot every
  // `every` steps, for backward().
  int record(int nsteps, int every) {
    if (!uploaded_) return fail(FLUID_ERR_STATE, "no state uploaded");
    if (nsteps < 1 || every < 1) return fail(FLUID_ERR_INVALID_ARGUMENT, "nsteps and checkpoint interval must be >= 1");
    int rc = synchronize();
    if (rc) return rc;
    checkpoints_.clear();
    const int segs = (nsteps + every - 1) / every;
    checkpoints_.resize(segs);
    tail_taped_ = false;
    if (static_cast<int>(tapes_.size()) < every) tapes_.resize(every);
    for (int seg = 0; seg < segs; ++seg) {
      const int t0 = seg * every, t1 = std::min(nsteps, t0 + every);
      if ((rc = snap_save(checkpoints_[seg]))) return rc;
      if (seg + 1 < segs) {
        if ((rc = step(t1 - t0))) return rc;  // one synchronisation per segment
      } else {
        // The last segment is taped as it runs: backward() reverses it first
        // and needs no recomputation for it.
        for (int t = t0; t < t1; ++t)
          if ((rc = taped_step(tapes_[t - t0]))) return rc;
      }
    }
    if ((rc = snap_save(final_))) return rc;
    rec_steps_ = nsteps;
    rec_every_ = every;
    tail_taped_ = true;
    return FLUID_OK;
  }

  // Back-propagates the cotangent of the final recorded state to the state
  // record() started from: each checkpoint segment is re-run forward to get
  // its step inputs, then stepped back in reverse. Leaves the solver at the
  // final state.
  int backward(const float* gpf, const float* gvf, float* gpi, float* gvi, float* gvisc, int memory) {
    if (rec_steps_ == 0) return fail(FLUID_ERR_STATE, "record() first");
    if (!gpf || !gvf || !gpi || !gvi) return fail(FLUID_ERR_INVALID_ARGUMENT, "null cotangent");
    int rc = synchronize();
    if (rc) return rc;
    if ((rc = ensure_adjoint_buffers())) return rc;
    const size_t m3 = 3 * static_cast<size_t>(n_);
    const size_t b = m3 * sizeof(float);
    float* cur[2] = {a_io_.p, a_io_.p + m3};
    float* nxt[2] = {a_io_.p + 2 * m3, a_io_.p + 3 * m3};
    const cudaMemcpyKind in = memory == FLUID_MEMORY_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
    cudaMemcpy(cur[0], gpf, b, in);
    cudaMemcpy(cur[1], gvf, b, in);
    std::vector<double> total(S_, 0.0), gc;
    const int segs = static_cast<int>(checkpoints_.size());
    if (static_cast<int>(tapes_.size()) < rec_every_) tapes_.resize(rec_every_);
    for (int seg = segs - 1; seg >= 0; --seg) {
      const int t0 = seg * rec_every_;
      const int t1 = std::min(rec_steps_, t0 + rec_every_);
      if (seg == segs - 1 && tail_taped_) {
        tail_taped_ = false;  // taped by record(); the tapes are reused below
      } else {
        if ((rc = snap_load(checkpoints_[seg]))) return rc;
        for (int t = t0; t < t1; ++t)  // recompute the segment once, taping every step
          if ((rc = taped_step(tapes_[t - t0]))) return rc;
      }
      for (int t = t1 - 1; t >= t0; --t) {
        if ((rc = tape_adjoint(tapes_[t - t0], cur[0], cur[1], nxt[0], nxt[1], gc))) return rc;
        for (int sc = 0; sc < S_; ++sc) total[sc] += gc[sc];
        std::swap(cur[0], nxt[0]);
        std::swap(cur[1], nxt[1]);
      }
    }
    if ((rc = snap_load(final_))) return rc;
    const cudaMemcpyKind out = memory == FLUID_MEMORY_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
    cudaMemcpy(gpi, cur[0], b, out);
    cudaMemcpy(gvi, cur[1], b, out);
    if (gvisc)
      for (int sc = 0; sc < S_; ++sc) gvisc[sc] = static_cast<float>(total[sc]);
    return FLUID_OK;
  }

  // ---- Frame output -------------------------------------------------------

  int frame_begin(int slot, float* hpos, float* hvel) {
    if (slot < 0 || slot > 1 || !hpos) return fail(FLUID_ERR_INVALID_ARGUMENT, "bad frame slot or buffer");
    if (!uploaded_) return fail(FLUID_ERR_STATE, "no state uploaded");
    int rc = synchronize();  // a pending step may still be re-run
    if (rc) return rc;
    const size_t n = static_cast<size_t>(std::max(n_, 1));
    if (!copy_stream_ && cudaStreamCreateWithFlags(&copy_stream_, cudaStreamNonBlocking) != cudaSuccess)
      return cuda_fail("copy stream");
    for (int k = 0; k < 2; ++k) {
      if (!frame_gather_[k] && (cudaEventCreateWithFlags(&frame_gather_[k], cudaEventDisableTiming) ||
                                cudaEventCreateWithFlags(&frame_done_[k], cudaEventDisableTiming)))
        return cuda_fail("frame events");
    }
    if (frame_stage_[slot].n != 6 * n && frame_stage_[slot].alloc(6 * n))
      return fail(FLUID_ERR_OUT_OF_MEMORY, "frame staging");
    if (frame_busy_[slot] && cudaEventSynchronize(frame_done_[slot]) != cudaSuccess) return cuda_fail("frame");
    if (n_ == 0) return FLUID_OK;
    float* st = frame_stage_[slot].p;
    const size_t m = static_cast<size_t>(n_);
    if (enqueue_download(x_[parity_].p, v_[parity_].p, slot_[parity_].p, st, st + m, st + 2 * m, st + 3 * m,
                         st + 4 * m, st + 5 * m, n_, stream_) != cudaSuccess)
      return cuda_fail("frame gather");
    cudaEventRecord(frame_gather_[slot], stream_);
    cudaStreamWaitEvent(copy_stream_, frame_gather_[slot], 0);
    cudaMemcpyAsync(hpos, st, 3 * m * sizeof(float), cudaMemcpyDeviceToHost, copy_stream_);
    if (hvel) cudaMemcpyAsync(hvel, st + 3 * m, 3 * m * sizeof(float), cudaMemcpyDeviceToHost, copy_stream_);
    if (cudaEventRecord(frame_done_[slot], copy_stream_) != cudaSuccess) return cuda_fail("frame copy");
    frame_busy_[slot] = true;
    return FLUID_OK;
  }

  int frame_wait(int slot) {
    if (slot < 0 || slot > 1) return fail(FLUID_ERR_INVALID_ARGUMENT, "bad frame slot");
    if (!frame_busy_[slot]) return FLUID_OK;
    if (cudaEventSynchronize(frame_done_[slot]) != cudaSuccess) return cuda_fail("frame wait");
    frame_busy_[slot] = false;
    return FLUID_OK;
  }

  int get_tuning(int32_t* unroll, int32_t* block, int kernels) {
    for (int k = 0; k < kernels && k < FLUID_KERNEL_COUNT; ++k) {
      if (unroll) unroll[k] = plan_.unroll[k];
      if (block) block[k] = plan_.block[k];
    }
    return FLUID_OK;
  }

  int set_tuning(const int32_t* unroll, const int32_t* block, int kernels) {
    for (int k = 0; k < kernels && k < FLUID_KERNEL_COUNT; ++k) {
      if (unroll && !(unroll[k] == 1 || unroll[k] == 2 || unroll[k] == 4 || unroll[k] == 8))
        return fail(FLUID_ERR_INVALID_ARGUMENT, "unroll must be 1, 2, 4 or 8");
      if (block && !(block[k] == 128 || block[k] == 256 || block[k] == 512))
        return fail(FLUID_ERR_INVALID_ARGUMENT, "block must be 128, 256 or 512");
    }
    int rc = synchronize();
    if (rc) return rc;
    for (int k = 0; k < kernels && k < FLUID_KERNEL_COUNT; ++k) {
      if (unroll && tunable_unroll(k)) plan_.unroll[k] = unroll[k];
      if (block && tunable_block(k)) plan_.block[k] = block[k];
    }
    invalidate_graphs();
    return FLUID_OK;
  }

  int get_lanes(int32_t* lanes, int kernels) {
    if (!lanes) return fail(FLUID_ERR_INVALID_ARGUMENT, "null lanes");
    for (int k = 0; k < kernels && k < FLUID_KERNEL_COUNT; ++k) lanes[k] = plan_.lanes[k];
    return FLUID_OK;
  }

  int set_lanes(const int32_t* lanes, int kernels) {
    if (!lanes) return fail(FLUID_ERR_INVALID_ARGUMENT, "null lanes");
    for (int k = 0; k < kernels && k < FLUID_KERNEL_COUNT; ++k) {
      if (!(lanes[k] == 1 || lanes[k] == 2 || lanes[k] == 4 || lanes[k] == 8))
        return fail(FLUID_ERR_INVALID_ARGUMENT, "lanes per particle must be 1, 2, 4 or 8");
      if (lanes[k] != 1 && !tunable_unroll(k))
        return fail(FLUID_ERR_INVALID_ARGUMENT, "only the neighbour-list passes take several lanes per particle");
    }
    int rc = synchronize();
    if (rc) return rc;
    for (int k = 0; k < kernels && k < FLUID_KERNEL_COUNT; ++k) plan_.lanes[k] = lanes[k];
    invalidate_graphs();
    return FLUID_OK;
  }

  int kernel_times(double* ms, int64_t* launches, int kernels, int reset) {
    for (int k = 0; k < kernels && k < FLUID_KERNEL_COUNT; ++k) {
      if (ms) ms[k] = stage_ms_[k];
      if (launches) launches[k] = stage_launches_[k];
    }
    if (reset) {
      std::fill(std::begin(stage_ms_), std::end(stage_ms_), 0.0);
      std::fill(std::begin(stage_launches_), std::end(stage_launches_), 0ll);
    }
    return FLUID_OK;
  }

  int get_time(int scene, float* t) {
    if (scene < 0 || scene >= S_ || !t) return fail(FLUID_ERR_INVALID_ARGUMENT, "bad scene");
    int rc = synchronize();
    if (rc) return rc;
    *t = times_[scene];
    return FLUID_OK;
  }

  int set_time(int scene, float t) {
    if (scene < 0 || scene >= S_) return fail(FLUID_ERR_INVALID_ARGUMENT, "bad scene");
    int rc = synchronize();
    if (rc) return rc;
    times_[scene] = t;
    return FLUID_OK;
  }

  int stats(fluid_stats* out) {
    if (!out) return fail(FLUID_ERR_INVALID_ARGUMENT, "null stats");
    int rc = synchronize();
    if (rc) return rc;
    out->particles = n_;
    out->steps = steps_;
    out->neighbor_pairs = last_pairs_;
    out->neighbor_max = last_max_;
    out->grid_cells = last_cells_;
    out->neighbor_capacity = nbr_cap_;
    out->grid_capacity = grid_cap_;
    out->regrows = regrows_;
    out->kernel_launches = launches_;
    return FLUID_OK;
  }

  int read_debug(int what, void* out, int64_t capacity) {
    if (!uploaded_ || steps_ == 0) return fail(FLUID_ERR_STATE, "no completed step");
    int rc = synchronize();
    if (rc) return rc;
    const int n = n_;
    const int64_t need = (what == FLUID_DEBUG_CELL_KEYS) ? 3ll * n : n;
    if (capacity < need || !out) return fail(FLUID_ERR_INVALID_ARGUMENT, "debug buffer too small");
    if (n == 0) return FLUID_OK;
    // Current parity holds the last step's output; keys/vals/cnt/lambda/rho
    // are the last step's scratch.
    std::vector<int> slot(n);
    if (cudaMemcpy(slot.data(), slot_[parity_].p, n * sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
      return cuda_fail("debug read");
    DevStatus st;
    cudaMemcpy(&st, status_.p, sizeof(st), cudaMemcpyDeviceToHost);
    const int npass = last_npass();
    if (what == FLUID_DEBUG_CELL_KEYS || what == FLUID_DEBUG_SORTED_ORDER) {
      std::vector<uint32_t> keys(n);
      std::vector<int> vals(n);
      cudaMemcpy(keys.data(), keys_[npass & 1].p, n * sizeof(uint32_t), cudaMemcpyDeviceToHost);
      if (npass)
        cudaMemcpy(vals.data(), vals_[npass & 1].p, n * sizeof(int), cudaMemcpyDeviceToHost);
      else
        for (int s = 0; s < n; ++s) vals[s] = s;
      std::vector<GridInfo> grid(S_);
      cudaMemcpy(grid.data(), grid_.p, S_ * sizeof(GridInfo), cudaMemcpyDeviceToHost);
      if (what == FLUID_DEBUG_SORTED_ORDER) {
        int32_t* o = static_cast<int32_t*>(out);
        for (int s = 0; s < n; ++s) o[s] = vals[s] - sc_host_[scene_of(vals[s])].first_slot;
      } else {
        int32_t* o = static_cast<int32_t*>(out);
        for (int s = 0; s < n; ++s) {
          const int orig = vals[s];
          const GridInfo& g = grid[scene_of(orig)];
          const long long l = static_cast<long long>(keys[s]) - g.base;
          const long long yz = static_cast<long long>(g.dimy) * g.dimz;
          o[3 * orig + 0] = g.minx + static_cast<int>(l / yz);
          o[3 * orig + 1] = g.miny + static_cast<int>((l % yz) / g.dimz);
          o[3 * orig + 2] = g.minz + static_cast<int>(l % g.dimz);
        }
      }
      return FLUID_OK;
    }
    std::vector<int32_t> buf(n);
    const void* src = nullptr;
    if (what == FLUID_DEBUG_NEIGHBOR_COUNTS) src = cnt_.p;
    else if (what == FLUID_DEBUG_RHO) src = rho_[parity_].p;
    else if (what == FLUID_DEBUG_LAMBDA) src = lambda_.p;
    else return fail(FLUID_ERR_INVALID_ARGUMENT, "unknown debug record");
    cudaMemcpy(buf.data(), src, n * sizeof(int32_t), cudaMemcpyDeviceToHost);
    int32_t* o = static_cast<int32_t*>(out);
    for (int orig = 0; orig < n; ++orig) o[orig] = buf[slot[orig]];
    return FLUID_OK;
  }

  const char* last_error() const { return err_.c_str(); }

 private:
  int fail(int code, const std::string& msg) {
    err_ = msg;
    return code;
  }
  int cuda_fail(const char* what) {
    cudaError_t e = cudaGetLastError();
    err_ = std::string(what) + ": " + cudaGetErrorString(e);
    if (e == cudaErrorMemoryAllocation) return FLUID_ERR_OUT_OF_MEMORY;
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return FLUID_ERR_NO_DEVICE;
    return FLUID_ERR_CUDA;
  }

  int synchronize_quiet() {
    if (stream_) cudaStreamSynchronize(stream_);
    pending_ = 0;
    return FLUID_OK;
  }

  void build_scene_consts() {
    sc_host_.resize(S_);
    long long first = 0;
    for (int s = 0; s < S_; ++s) {
      sc_host_[s] = make_scene_const(params_[s], static_cast<int>(first), static_cast<int>(counts_[s]));
      first += counts_[s];
    }
  }

  int scene_of(int orig) const {
    int lo = 0, hi = S_ - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) / 2;
      if (sc_host_[mid].first_slot <= orig) lo = mid; else hi = mid - 1;
    }
    return lo;
  }

  int last_npass() const { return last_npass_; }

  void make_plan() {
    plan_.iterations = params_[0].solver_iterations;
    plan_.xsph = plan_.vorticity = plan_.restitution = false;
    for (const auto& c : sc_host_) {
      plan_.xsph |= c.xsph_on != 0;
      plan_.vorticity |= c.vort_on != 0;
      plan_.restitution |= c.rest_on != 0;
    }
    plan_.radix_passes = std::max(1, (bits_for(grid_cap_) + plan_.radix_bits - 1) / plan_.radix_bits);
    plan_.scorr_pow = shared_scorr_pow(sc_host_.data(), S_);
    plan_.ieee_sqrt = false;
    for (const auto& c : sc_host_) plan_.ieee_sqrt |= c.exact_sqrt != 0;
  }

  void advance_times(int steps) {
    for (int k = 0; k < steps; ++k)
      for (int s = 0; s < S_; ++s) times_[s] += params_[s].dt;  // core.cpp:614
  }

  void commit_steps(int done) {
    advance_times(done);
    steps_ += done;
    parity_ = (parity_ + done) & 1;
  }

  StepArgs args(int par) {
    StepArgs a;
    std::memset(&a, 0, sizeof(a));
    a.x_old = x_[par].p;
    a.v_old = v_[par].p;
    a.slot_old = slot_[par].p;
    a.rho_old = rho_[par].p;
    a.x = x_[par ^ 1].p;
    a.v = v_[par ^ 1].p;
    a.v2 = v2_.p;
    a.slot = slot_[par ^ 1].p;
    a.p[0] = p_[0].p;
    a.p[1] = p_[1].p;
    a.omega = omega_.p;
    a.pl = pl_.p;
    a.lambda = lambda_.p;
    a.rho = rho_[par ^ 1].p;
    a.keys[0] = keys_[0].p;
    a.keys[1] = keys_[1].p;
    a.vals[0] = vals_[0].p;
    a.vals[1] = vals_[1].p;
    a.look = look_.p;
    a.live = live_.p;
    a.radix_next = radix_next_.p;
    a.digit_total = digit_total_.p;
    a.table = table_.p;
    a.cnt = cnt_.p;
    a.depth = depth_.p;
    a.slice_fmt = ovf_.p;
    a.list16 = 1;
    a.wbase = wbase_.p;
    a.nbr = nbr_.p;
    a.bmin = bmin_.p;
    a.bmax = bmax_.p;
    a.grid = grid_.p;
    a.status = status_.p;
    a.sc = sc_.p;
    a.n = n_;
    a.scenes = S_;
    a.tiles = tiles_;
    a.warps = warps_;
    a.grid_capacity = grid_cap_;
    a.nbr_capacity = nbr_cap_;
    return a;
  }

  LaunchMarks marks(int par, bool capturing) {
    LaunchMarks m;
    m.on = profiling_;
    m.stream = stream_;
    m.capturing = capturing;
    m.events = &events_[par];
    m.stages = &stages_[par];
    return m;
  }

  int launch_one() {
    const int par = (parity_ + pending_) & 1;
    if (use_graphs_) {
      if (!graphs_valid_) {
        int rc = build_graphs();
        if (rc) return rc;
      }
      // The box from the upload serves only the step right after it; a
      // step re-run after regrowth recomputes it.
      cudaGraphExec_t& split = split_exec_[2 * par + (bounds_ready_ ? 1 : 0)];
      if (split_on_ && !split) {
        split_.bounds_done = bounds_ready_;
        int rc = capture(par, &split_, &split);
        split_.bounds_done = false;
        if (rc) return rc;
      }
      if (cudaGraphLaunch(split_on_ ? split : exec_[par], stream_) != cudaSuccess)
        return cuda_fail("graph launch");
      launches_ += launches_per_step_ - ((split_on_ && bounds_ready_) ? 1 : 0);
    } else {
      LaunchMarks m = marks(par, false);
      split_.bounds_done = split_on_ && bounds_ready_;
      const cudaError_t e = enqueue_step(args(par), plan_, stream_, m, nullptr, split_on_ ? &split_ : nullptr);
      split_.bounds_done = false;
      if (e != cudaSuccess) return cuda_fail("launch");
      launches_ += m.launches;
      launches_per_step_ = m.launches;
      marks_used_[par] = m.next;
    }
    bounds_ready_ = false;
    ++pending_;
    return FLUID_OK;
  }

  // Captures one step of parity `par` (with the result write-out when dl).
  int capture(int par, const StepDownload* dl, cudaGraphExec_t* out) {
    cudaGraph_t g = nullptr;
    if (cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
      return cuda_fail("begin capture");
    LaunchMarks m = marks(par, true);
    cudaError_t e = enqueue_step(args(par), plan_, stream_, m, nullptr, dl);
    cudaError_t e2 = cudaStreamEndCapture(stream_, &g);
    if (e != cudaSuccess || e2 != cudaSuccess || !g) return cuda_fail("capture");
    if (cudaGraphInstantiate(out, g, 0) != cudaSuccess) {
      cudaGraphDestroy(g);
      return cuda_fail("graph instantiate");
    }
    cudaGraphDestroy(g);
    if (!dl) {
      launches_per_step_ = m.launches;
      marks_used_[par] = m.next;
    }
    return FLUID_OK;
  }

  int build_graphs() {
    destroy_graphs();
    for (int par = 0; par < 2; ++par) {
      int rc = capture(par, nullptr, &exec_[par]);
      if (rc) return rc;
    }
    graphs_valid_ = true;
    return FLUID_OK;
  }

  void destroy_graphs() {
    for (auto& e : exec_) {
      if (e) cudaGraphExecDestroy(e);
      e = nullptr;
    }
    for (auto& e : split_exec_) {
      if (e) cudaGraphExecDestroy(e);
      e = nullptr;
    }
    graphs_valid_ = false;
  }
  void invalidate_graphs() { destroy_graphs(); }

  void destroy_events() {
    for (auto& v : events_)
      for (auto& e : v) cudaEventDestroy(e);
  }

  void accumulate_profile(int par) {
    const int used = marks_used_[par];
    for (int k = 1; k < used; ++k) {
      float ms = 0.0f;
      if (cudaEventElapsedTime(&ms, events_[par][k - 1], events_[par][k]) == cudaSuccess) {
        const int st = stages_[par][k];
        stage_ms_[st] += ms;
        stage_launches_[st] += 1;
      }
    }
  }

  // The list build's staged rows follow the lists: raised (never lowered
  // while the lists fit) to cover the longest list of a step when that fits
  // kMaxStageRows, so a scene whose longest list sits just above the default
  // (the 4,096-particle dam break: 35-40) has its lists staged whole instead
  // of scanned a second time; back to the default once lists outgrow
  // it (a collapse, where the second scan runs anyway and a smaller stage
  // leaves the L1 more room for the candidates).
  void adapt_stage_rows(int longest) {
    int rows = plan_.stage_rows;
    if (longest > kMaxStageRows) rows = kStageRowsDefault;
    else if (longest > rows) rows = std::min(kMaxStageRows, static_cast<int>(round_up(longest + 2, 4)));
    if (rows == plan_.stage_rows) return;
    plan_.stage_rows = rows;
    invalidate_graphs();
  }

  // Grows the list capacity before a step needs it. After a step that
  // succeeded, nothing is in flight: if this step's lists, times their
  // growth over the previous step's (1-4x) and a quarter more, would not fit,
  // the buffer is reallocated now, to at least twice its size. A neighbourhood that grows step after step
  // (a collapse) then rarely fails a step, whose re-run after a regrow costs
  // as much as the step itself. An allocation that fails here keeps the old
  // capacity; the step that outgrows it regrows as before.
  int grow_ahead(unsigned long long used) {
    const unsigned long long prev = last_list_ints_;
    last_list_ints_ = used;
    if (prev == 0 || used == 0) return FLUID_OK;
    const double ratio = std::min(4.0, std::max(1.0, double(used) / double(prev)));
    const double want = double(used) * ratio * 1.25;
    if (want <= double(nbr_cap_)) return FLUID_OK;
    const long long old = nbr_cap_;
    // At least double: a reallocation of several GB costs tens of ms, so the
    // capacity grows geometrically rather than to each step's projection.
    const long long cap = round_up(std::max(static_cast<long long>(std::ceil(want)), 2 * old), 32);
    nbr_.release();
    if (nbr_.alloc(static_cast<size_t>(cap)) != cudaSuccess) {
      cudaGetLastError();  // the failed allocation is not an error of the solver
      if (nbr_.alloc(static_cast<size_t>(old)) != cudaSuccess) {
        nbr_cap_ = 0;
        return fail(FLUID_ERR_OUT_OF_MEMORY, "neighbour lists of " + std::to_string(old) + " entries");
      }
      return FLUID_OK;
    }
    nbr_cap_ = cap;
    ++grows_ahead_;
    make_plan();
    invalidate_graphs();
    return FLUID_OK;
  }

  int grow(unsigned long long need_grid, unsigned long long need_nbr) {
    cudaStreamSynchronize(stream_);
    float f = 1.5f;
    for (const auto& p : params_) f = std::max(f, p.neighbor_reserve_factor);
    bool changed = false;
    if (need_grid > static_cast<unsigned long long>(grid_cap_)) {
      long long cap = static_cast<long long>(std::ceil(double(need_grid) * f));
      cap = std::min<long long>(cap, (1ll << 31) - 1);
      if (table_.alloc(static_cast<size_t>(cap)) != cudaSuccess) return fail(FLUID_ERR_OUT_OF_MEMORY, "cell table");
      cudaMemsetAsync(table_.p, 0, table_.n * sizeof(int2), stream_);
      cudaMemsetAsync(look_.p, 0, look_.n * sizeof(unsigned long long), stream_);  // tag 0: never current
      grid_cap_ = cap;
      changed = true;
    }
    if (need_nbr > static_cast<unsigned long long>(nbr_cap_)) {
      const long long cap = round_up(static_cast<long long>(std::ceil(double(need_nbr) * f)), 32);
      nbr_.release();
      if (nbr_.alloc(static_cast<size_t>(cap)) != cudaSuccess) {
        nbr_cap_ = 0;
        return fail(FLUID_ERR_OUT_OF_MEMORY, "neighbour lists of " + std::to_string(cap) + " entries");
      }
      nbr_cap_ = cap;
      changed = true;
    }
    if (!changed) return fail(FLUID_ERR_CAPACITY, "capacity error without growth");
    make_plan();
    invalidate_graphs();
    return FLUID_OK;
  }

  struct Snap {
    DBuf<float4> x, v;
    DBuf<int> slot;
    DBuf<float> rho;
    std::vector<float> times;
    long long steps = 0;
  };

  int snap_save(Snap& sn) {
    const size_t n = static_cast<size_t>(std::max(n_, 1));
    if (sn.x.n != n) {
      if (sn.x.alloc(n) || sn.v.alloc(n) || sn.slot.alloc(n) || sn.rho.alloc(n))
        return fail(FLUID_ERR_OUT_OF_MEMORY, "snapshot");
    }
    cudaMemcpyAsync(sn.x.p, x_[parity_].p, n * sizeof(float4), cudaMemcpyDeviceToDevice, stream_);
    cudaMemcpyAsync(sn.v.p, v_[parity_].p, n * sizeof(float4), cudaMemcpyDeviceToDevice, stream_);
    cudaMemcpyAsync(sn.slot.p, slot_[parity_].p, n * sizeof(int), cudaMemcpyDeviceToDevice, stream_);
    cudaMemcpyAsync(sn.rho.p, rho_[parity_].p, n * sizeof(float), cudaMemcpyDeviceToDevice, stream_);
    sn.times = times_;
    sn.steps = steps_;
    return cudaStreamSynchronize(stream_) == cudaSuccess ? FLUID_OK : cuda_fail("snapshot");
  }

  int snap_load(const Snap& sn) {
    const size_t n = static_cast<size_t>(std::max(n_, 1));
    cudaMemcpyAsync(x_[parity_].p, sn.x.p, n * sizeof(float4), cudaMemcpyDeviceToDevice, stream_);
    cudaMemcpyAsync(v_[parity_].p, sn.v.p, n * sizeof(float4), cudaMemcpyDeviceToDevice, stream_);
    cudaMemcpyAsync(slot_[parity_].p, sn.slot.p, n * sizeof(int), cudaMemcpyDeviceToDevice, stream_);
    cudaMemcpyAsync(rho_[parity_].p, sn.rho.p, n * sizeof(float), cudaMemcpyDeviceToDevice, stream_);
    times_ = sn.times;
    steps_ = sn.steps;
    return cudaStreamSynchronize(stream_) == cudaSuccess ? FLUID_OK : cuda_fail("restore");
  }

  // One step's forward internals and neighbour lists, for the adjoint.
  struct Tape {
    DBuf<float4> x0, p, q, omega;
    DBuf<float> lam, rho;
    DBuf<int> cnt, nbr;
    DBuf<long long> wbase;
    size_t n = 0;
    int k = -1;
  };

  // Runs one step from the current state (advancing it like step(1)) and
  // tapes what the adjoint needs. Capacity overflows regrow and re-run.
  int taped_step(Tape& tp) {
    const size_t n = static_cast<size_t>(std::max(n_, 1));
    const int k = plan_.iterations;
    if (tp.n != n || tp.k != k) {
      const size_t kk = static_cast<size_t>(std::max(k, 1));
      if (tp.x0.alloc(n) || tp.p.alloc((k + 1) * n) || tp.q.alloc(kk * n) || tp.lam.alloc(kk * n) ||
          tp.rho.alloc(n) || tp.omega.alloc(n) || tp.cnt.alloc(n) ||
          tp.wbase.alloc(static_cast<size_t>(warps_) + 1)) {
        tp.n = 0;
        return fail(FLUID_ERR_OUT_OF_MEMORY, "adjoint tape");
      }
      tp.n = n;
      tp.k = k;
    }
    for (;;) {
      StepRecord rec;
      rec.x0 = tp.x0.p;
      rec.p = tp.p.p;
      rec.q = tp.q.p;
      rec.lambda = tp.lam.p;
      rec.rho = tp.rho.p;
      rec.omega = tp.omega.p;
      LaunchMarks m;
      if (enqueue_step(args(parity_), plan_, stream_, m, &rec) != cudaSuccess) return cuda_fail("taped step");
      launches_ += m.launches;
      if (cudaStreamSynchronize(stream_) != cudaSuccess) return cuda_fail("taped step");
      DevStatus st;
      cudaMemcpy(&st, status_.p, sizeof(st), cudaMemcpyDeviceToHost);
      enqueue_reset(status_.p, bmin_.p, bmax_.p, S_, stream_);
      if (st.err == FLUID_ERR_CAPACITY) {
        int rc = grow(st.need_grid, st.cursor);
        if (rc) return rc;
        ++regrows_;
        continue;
      }
      if (st.err) {
        cudaStreamSynchronize(stream_);
        return fail(st.err, "taped step failed");
      }
      const size_t len = static_cast<size_t>(st.cursor);
      if (tp.nbr.n < len && tp.nbr.alloc(len + len / 4 + 32)) return fail(FLUID_ERR_OUT_OF_MEMORY, "adjoint tape");
      cudaMemcpyAsync(tp.nbr.p, nbr_.p, len * sizeof(int), cudaMemcpyDeviceToDevice, stream_);
      cudaMemcpyAsync(tp.cnt.p, cnt_.p, n * sizeof(int), cudaMemcpyDeviceToDevice, stream_);
      cudaMemcpyAsync(tp.wbase.p, wbase_.p, (static_cast<size_t>(warps_) + 1) * sizeof(long long),
                      cudaMemcpyDeviceToDevice, stream_);
      last_pairs_ = static_cast<long long>(st.pairs);
      last_max_ = st.nbr_max;
      last_cells_ = static_cast<int>(st.total_cells);
      last_npass_ = st.npass;
      commit_steps(1);
      return FLUID_OK;
    }
  }

  // Adjoint kernels over one tape; cotangents on the device (3n blocks).
  int tape_adjoint(const Tape& tp, const float* gpo, const float* gvo, float* gpi, float* gvi,
                   std::vector<double>& gc) {
    StepArgs sa = args(parity_);
    sa.cnt = tp.cnt.p;
    sa.nbr = tp.nbr.p;
    sa.wbase = tp.wbase.p;
    AdjArgs aa;
    aa.s = sa;
    aa.rec.x0 = tp.x0.p;
    aa.rec.p = tp.p.p;
    aa.rec.q = tp.q.p;
    aa.rec.lambda = tp.lam.p;
    aa.rec.rho = tp.rho.p;
    aa.rec.omega = tp.omega.p;
    aa.iters = tp.k;
    aa.vorticity = plan_.vorticity ? 1 : 0;
    aa.v3 = a_v3_.p;
    aa.dv = a_dv_.p;
    aa.gv4 = a_gv4_.p;
    aa.eb = a_eb_.p;
    aa.obd = a_obd_.p;
    aa.ob = a_ob_.p;
    aa.v2 = a_v2_.p;
    aa.gx = a_gx_.p;
    aa.gv = a_gv_.p;
    aa.gv3 = a_gv3_.p;
    aa.gp = a_gp_.p;
    aa.gd = a_gd_.p;
    aa.gx0 = a_gx0_.p;
    aa.aux = a_aux_.p;
    aa.pg = a_pg_.p;
    aa.grho = a_grho_.p;
    aa.cc = a_cc_.p;
    aa.g_pos_out = gpo;
    aa.g_vel_out = gvo;
    aa.g_pos_in = gpi;
    aa.g_vel_in = gvi;
    if (enqueue_adjoint(aa, stream_) != cudaSuccess) return cuda_fail("adjoint launch");
    launches_ += 4 + 3ll * tp.k + (plan_.vorticity ? 2 : 0);
    std::vector<float> cc(n_);
    if (cudaMemcpyAsync(cc.data(), a_cc_.p, sizeof(float) * n_, cudaMemcpyDeviceToHost, stream_) != cudaSuccess ||
        cudaStreamSynchronize(stream_) != cudaSuccess)
      return cuda_fail("adjoint");
    gc.assign(S_, 0.0);
    for (int sc = 0; sc < S_; ++sc) {
      double acc = 0.0;
      for (int i = sc_host_[sc].first_slot; i < sc_host_[sc].first_slot + sc_host_[sc].count; ++i) acc += cc[i];
      gc[sc] = acc;
    }
    return FLUID_OK;
  }

  int ensure_adjoint_buffers() {
    const size_t n = static_cast<size_t>(std::max(n_, 1));
    if (adj_n_ == n) return FLUID_OK;
    bool ok = a_v2_.alloc(n) == cudaSuccess && a_gx_.alloc(n) == cudaSuccess && a_gv_.alloc(n) == cudaSuccess &&
              a_gv3_.alloc(n) == cudaSuccess && a_gp_.alloc(n) == cudaSuccess && a_gd_.alloc(n) == cudaSuccess &&
              a_gx0_.alloc(n) == cudaSuccess && a_aux_.alloc(n) == cudaSuccess && a_pg_.alloc(n) == cudaSuccess &&
              a_grho_.alloc(n) == cudaSuccess && a_cc_.alloc(n) == cudaSuccess && a_io_.alloc(12 * n) == cudaSuccess &&
              a_v3_.alloc(n) == cudaSuccess && a_dv_.alloc(n) == cudaSuccess && a_gv4_.alloc(n) == cudaSuccess &&
              a_eb_.alloc(n) == cudaSuccess && a_obd_.alloc(n) == cudaSuccess && a_ob_.alloc(n) == cudaSuccess;
    if (!ok) {
      adj_n_ = 0;
      return fail(FLUID_ERR_OUT_OF_MEMORY, "adjoint buffers");
    }
    adj_n_ = n;
    return FLUID_OK;
  }

  DBuf<float4> a_v2_, a_gx_, a_gv_, a_gv3_, a_gp_, a_gd_, a_gx0_, a_aux_, a_pg_, a_v3_, a_dv_, a_gv4_, a_eb_, a_obd_, a_ob_;
  DBuf<float> a_grho_, a_cc_, a_io_;
  size_t adj_n_ = 0;
  std::vector<Tape> tapes_;
  std::vector<Snap> checkpoints_;
  Snap final_;
  int rec_steps_ = 0, rec_every_ = 1;
  bool tail_taped_ = false;  // tapes_ hold record()'s last segment

  cudaStream_t copy_stream_ = nullptr;
  cudaEvent_t frame_gather_[2] = {nullptr, nullptr}, frame_done_[2] = {nullptr, nullptr};
  bool frame_busy_[2] = {false, false};
  DBuf<float> frame_stage_[2];

  int device_;
  cudaStream_t own_ = nullptr, stream_ = nullptr;
  int S_ = 0, n_ = 0, warps_ = 0, tiles_ = 1;
  std::vector<fluid_params> params_;
  std::vector<int64_t> counts_;
  std::vector<SceneConst> sc_host_;
  std::vector<float> times_;
  bool uploaded_ = false;
  int parity_ = 0, pending_ = 0;
  long long steps_ = 0, regrows_ = 0, launches_ = 0, launches_per_step_ = 0;
  long long grows_ahead_ = 0;              // list reallocations before a step needed them
  unsigned long long last_list_ints_ = 0;  // list ints the last completed step claimed
  long long last_pairs_ = 0;
  int last_max_ = 0, last_cells_ = 0, last_npass_ = 0;
  DBuf<float4> x_[2], v_[2], p_[2], v2_, omega_, pl_;
  DBuf<int> slot_[2], vals_[2], cnt_, depth_, ovf_, nbr_, bmin_, bmax_;
  DBuf<float> rho_[2], lambda_;
  DBuf<uint32_t> keys_[2], digit_total_;
  DBuf<unsigned long long> look_;
  DBuf<uint32_t> live_;
  DBuf<int> radix_next_;
  DBuf<long long> wbase_;
  DBuf<int2> table_;
  DBuf<GridInfo> grid_;
  DBuf<DevStatus> status_;
  DBuf<SceneConst> sc_;
  DevStatus* status_host_ = nullptr;
  cudaStream_t aux_ = nullptr;  // stateless step: positions written out beside the velocity passes
  StepDownload split_;
  bool split_on_ = false;
  DBuf<float*> targets_;          // the write-out's six destination arrays
  float** targets_host_ = nullptr;
  cudaGraphExec_t split_exec_[4] = {nullptr, nullptr, nullptr, nullptr};  // [2 * parity + box from upload]
  bool bounds_ready_ = false;  // the last upload added the predicted cells to the bounding box
  long long grid_cap_ = 0, nbr_cap_ = 0;
  StepPlan plan_;
  bool use_graphs_ = true, graphs_valid_ = false, profiling_ = false;
  cudaGraphExec_t exec_[2] = {nullptr, nullptr};
  std::vector<cudaEvent_t> events_[2];
  std::vector<int> stages_[2];
  int marks_used_[2] = {0, 0};
  double stage_ms_[FLUID_KERNEL_COUNT] = {};
  long long stage_launches_[FLUID_KERNEL_COUNT] = {};
  std::string err_;
};

}  // namespace fgb

struct fluid_solver {
  fgb::Solver impl;
  explicit fluid_solver(int d) : impl(d) {}
};

extern "C" {

void fluid_params_default(fluid_params* p) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  // core/include/fluid/core.h:12-43
  p->dt = 1.0f / 60.0f;
  p->density = 6000.0f;
  p->particle_mass = 0.0f;
  p->h = 0.0f;
  p->particle_radius = 0.01f;
  p->epsilon = 600.0f;
  p->solver_iterations = 4;
  p->neighbor_reserve_factor = 1.5f;
  p->use_uniform_grid = 1;
  p->enable_scorr = 0;
  p->enable_xsph = 0;
  p->enable_vorticity = 0;
  p->scorr_k = 0.00005f;
  p->scorr_n = 4;
  p->scorr_dq_coeff = 0.3f;
  p->visc_c = 0.0002f;
  p->plane_restitution = 0.0f;
  p->plane_friction = 0.0f;
  p->vort_epsilon = 0.5f;
  p->vort_norm_eps = 1e-6f;
  p->external_force[0] = 0.0f;
  p->external_force[1] = -9.8f;
  p->external_force[2] = 0.0f;
  p->plane_count = 0;
}

int fluid_gb300_version(void) { return FLUID_GB300_ABI_VERSION; }

int fluid_gb300_device_available(int* count, const char** error) {
  int n = 0;
  const cudaError_t e = cudaGetDeviceCount(&n);
  if (count) *count = 0;
  if (error) *error = nullptr;
  if (e == cudaErrorNoDevice) return 0;
  if (e != cudaSuccess) {
    if (error) *error = cudaGetErrorString(e);
    return 0;
  }
  if (count) *count = n;
  return n > 0 ? 1 : 0;
}

const char* fluid_status_string(int status) {
  switch (status) {
    case FLUID_OK: return "ok";
    case FLUID_ERR_INVALID_ARGUMENT: return "invalid argument";
    case FLUID_ERR_CUDA: return "CUDA error";
    case FLUID_ERR_CAPACITY: return "capacity exceeded";
    case FLUID_ERR_DOMAIN: return "grid domain too large";
    case FLUID_ERR_NONFINITE: return "non-finite position";
    case FLUID_ERR_NO_DEVICE: return "no CUDA device";
    case FLUID_ERR_OUT_OF_MEMORY: return "out of device memory";
    case FLUID_ERR_NOT_SUPPORTED: return "not supported";
    case FLUID_ERR_STATE: return "invalid call order";
    default: return "unknown status";
  }
}

int fluid_solver_create(fluid_solver** out, int device) {
  if (!out) return FLUID_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  int count = 0;
  if (!fluid_gb300_device_available(&count, nullptr)) return FLUID_ERR_NO_DEVICE;
  if (device < 0 || device >= count) return FLUID_ERR_INVALID_ARGUMENT;
  auto s = std::make_unique<fluid_solver>(device);
  const int rc = s->impl.init();
  if (rc) return rc;
  *out = s.release();
  return FLUID_OK;
}

void fluid_solver_destroy(fluid_solver* s) { delete s; }

#define FLUID_CHECK_SOLVER(s) \
  if (!(s)) return FLUID_ERR_INVALID_ARGUMENT

int fluid_solver_set_stream(fluid_solver* s, void* stream) {
  FLUID_CHECK_SOLVER(s);
  return s->impl.set_stream(stream);
}

int fluid_solver_configure(fluid_solver* s, int32_t scene_count, const fluid_params* params,
                           const int64_t* counts) {
  FLUID_CHECK_SOLVER(s);
  return s->impl.configure(scene_count, params, counts);
}

int fluid_solver_set_params(fluid_solver* s, const fluid_params* params) {
  FLUID_CHECK_SOLVER(s);
  if (!params) return FLUID_ERR_INVALID_ARGUMENT;
  return s->impl.set_params(params);
}

int fluid_solver_upload(fluid_solver* s, const float* px, const float* py, const float* pz, const float* vx,
                        const float* vy, const float* vz, int32_t memory) {
  FLUID_CHECK_SOLVER(s);
  return s->impl.upload(px, py, pz, vx, vy, vz, memory);
}

int fluid_solver_download(fluid_solver* s, float* px, float* py, float* pz, float* vx, float* vy, float* vz,
                          int32_t memory) {
  FLUID_CHECK_SOLVER(s);
  return s->impl.download(px, py, pz, vx, vy, vz, memory);
}

int fluid_solver_step(fluid_solver* s, int32_t nsteps) {
  FLUID_CHECK_SOLVER(s);
  return s->impl.step(nsteps);
}

int fluid_solver_step_async(fluid_solver* s, int32_t nsteps) {
  FLUID_CHECK_SOLVER(s);
  return s->impl.step_async(nsteps);
}

int fluid_solver_synchronize(fluid_solver* s) {
  FLUID_CHECK_SOLVER(s);
  return s->impl.synchronize();
}

int fluid_solver_set_graphs(fluid_solver* s, int32_t enable) {
  FLUID_CHECK_SOLVER(s);
  return s->impl.set_graphs(enable);
}

int fluid_solver_set_profiling(fluid_solver* s, int32_t enable) {
  FLUID_CHECK_SOLVER(s);
  return s->impl.set_profiling(enable);
}

int fluid_solver_kernel_times(fluid_solver* s, double* ms, int64_t* launches, int32_t kernels, int32_t reset) {
  FLUID_CHECK_SOLVER(s);
  return s->impl.kernel_times(ms, launches, kernels, reset);
}

const char* fluid_kernel_name(int kernel) {
  static const char* const names[FLUID_KERNEL_COUNT] = {
      "k_bounds", "k_grid_setup", "k_keys", "k_radix_digits", "k_radix_starts", "k_radix_onesweep",
      "k_reorder", "k_nbr_build", "k_nbr_overflow", "k_lambda", "k_delta",
      "k_commit", "k_xsph", "k_omega", "k_eta"};
  return (kernel >= 0 && kernel < FLUID_KERNEL_COUNT) ? names[kernel] : nullptr;
}

int fluid_solver_autotune(fluid_solver* s, int32_t trials) {
  FLUID_CHECK_SOLVER(s);
  return s->impl.autotune(trials);
}

int fluid_solver_get_tuning(fluid_solver* s, int32_t* unroll, int32_t* block, int32_t kernels) {
  FLUID_CHECK_SOLVER(s);
  return s->impl.get_tuning(unroll, block, kernels);
}

int fluid_solver_set_tuning(fluid_solver* s, const int32_t* unroll, const int32_t* block, int32_t kernels) {
  FLUID_CHECK_SOLVER(s);
  return s->impl.set_tuning(unroll, block, kernels);
}

int fluid_solver_get_lanes(fluid_solver* s, int32_t* lanes, int32_t kernels) {
  FLUID_CHECK_SOLVER(s);
  return s->impl.get_lanes(lanes, kernels);
}

int fluid_solver_set_lanes(fluid_solver* s, const int32_t* lanes, int32_t kernels) {
  FLUID_CHECK_SOLVER(s);
  return s->impl.set_lanes(lanes, kernels);
}

int fluid_solver_get_sort_bits(fluid_solver* s, int32_t* bits) {
  FLUID_CHECK_SOLVER(s);
  if (!bits) return FLUID_ERR_INVALID_ARGUMENT;
  *bits = s->impl.sort_bits();
  return FLUID_OK;
}

int fluid_solver_set_sort_bits(fluid_solver* s, int32_t bits) {
  FLUID_CHECK_SOLVER(s);
  return s->impl.set_sort_bits(bits);
}

int fluid_solver_step_backward(fluid_solver* s, const float* g_pos_out, const float* g_vel_out, float* g_pos_in,
                               float* g_vel_in, float* g_visc_c, int32_t memory) {
  FLUID_CHECK_SOLVER(s);
  return s->impl.step_backward(g_pos_out, g_vel_out, g_pos_in, g_vel_in, g_visc_c, memory);
}

int fluid_solver_record(fluid_solver* s, int32_t nsteps, int32_t checkpoint_every) {
  FLUID_CHECK_SOLVER(s);
  return s->impl.record(nsteps, checkpoint_every);
}

int fluid_solver_backward(fluid_solver* s, const float* g_pos_final, const float* g_vel_final, float* g_pos_initial,
                          float* g_vel_initial, float* g_visc_c, int32_t memory) {
  FLUID_CHECK_SOLVER(s);
  return s->impl.backward(g_pos_final, g_vel_final, g_pos_initial, g_vel_initial, g_visc_c, memory);
}

int fluid_solver_frame_begin(fluid_solver* s, int32_t slot, float* host_pos, float* host_vel) {
  FLUID_CHECK_SOLVER(s);
  return s->impl.frame_begin(slot, host_pos, host_vel);
}

int fluid_solver_frame_wait(fluid_solver* s, int32_t slot) {
  FLUID_CHECK_SOLVER(s);
  return s->impl.frame_wait(slot);
}

int fluid_solver_get_time(fluid_solver* s, int32_t scene, float* time) {
  FLUID_CHECK_SOLVER(s);
  return s->impl.get_time(scene, time);
}

int fluid_solver_set_time(fluid_solver* s, int32_t scene, float time) {
  FLUID_CHECK_SOLVER(s);
  return s->impl.set_time(scene, time);
}

int fluid_solver_get_stats(fluid_solver* s, fluid_stats* out) {
  FLUID_CHECK_SOLVER(s);
  return s->impl.stats(out);
}

int fluid_solver_read_debug(fluid_solver* s, int32_t what, void* host_out, int64_t capacity) {
  FLUID_CHECK_SOLVER(s);
  return s->impl.read_debug(what, host_out, capacity);
}

const char* fluid_solver_last_error(const fluid_solver* s) {
  return s ? s->impl.last_error() : "null solver";
}

int fluid_gb300_cuda_step(const fluid_params* params, int64_t count, float* px, float* py, float* pz, float* vx,
                          float* vy, float* vz, float* time) {
  if (!params || !time || count < 0) return FLUID_ERR_INVALID_ARGUMENT;
  if (count == 0) {  // cuda_stub.cu:766-769
    *time += params->dt;
    return FLUID_OK;
  }
  struct Cache {
    std::unique_ptr<fluid_solver> s;
    int64_t count = -1;
    int device = -1;
  };
  thread_local Cache cache;
  int device = 0;
  if (cudaGetDevice(&device) != cudaSuccess) return FLUID_ERR_NO_DEVICE;
  int rc;
  if (!cache.s || cache.count != count || cache.device != device) {
    cache.s.reset();
    fluid_solver* raw = nullptr;
    rc = fluid_solver_create(&raw, device);
    if (rc) return rc;
    cache.s.reset(raw);
    rc = cache.s->impl.configure(1, params, &count);
    if (rc) {
      cache.s.reset();
      return rc;
    }
    cache.count = count;
    cache.device = device;
  } else {
    rc = cache.s->impl.set_params(params);
    if (rc) return rc;
  }
  fgb::Solver& s = cache.s->impl;
  // The host arrays are read by copies left in flight: the step and the
  // download that follow on the same stream finish before this returns.
  if ((rc = s.upload(px, py, pz, vx, vy, vz, FLUID_MEMORY_HOST, false, true))) return rc;
  if ((rc = s.set_time(0, *time))) return rc;
  if ((rc = s.step_download_host(px, py, pz, vx, vy, vz))) return rc;
  return s.get_time(0, time);
}

}  // extern "C"

namespace fgb {

// Exported for the no-allocation entry point (pbf_noalloc.cu).
SceneConst scene_const_for(const fluid_params& p, int first, int count) { return make_scene_const(p, first, count); }

int params_status(const fluid_params& p) {
  std::string why;
  return validate_params(p, why);
}

}  // namespace fgb
