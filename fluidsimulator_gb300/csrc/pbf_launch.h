// Host-side launch interface of the PBF step kernels.
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "pbf_common.cuh"

namespace fgb {

// What one step launches; fixed for a configuration, so a captured graph of
// it stays valid until buffers are reallocated or the flags change.
// Staged list rows of the build: the default, and the most a block of
// kMaxStageBlock threads can stage in 48 KB of shared memory with a spare row.
constexpr int kStageRowsDefault = 36;
constexpr int kMaxStageBlock = 256;
constexpr int kMaxStageRows = 44;

constexpr int kDefaultListBlock = 128;  // threads per block of the list passes unless tuned
constexpr long long kFewParticles = 16384;   // at most this many in all: eight lanes in lambda and delta
constexpr long long kSomeParticles = 32768;  // at most this many: four

struct StepPlan {
  int iterations = 0;
  bool xsph = false;      // some scene runs XSPH
  bool vorticity = false; // some scene runs vorticity confinement
  bool restitution = false;
  int radix_passes = 1;   // passes launched (cover the grid capacity)
  int radix_bits = 9;     // digit width of the sort: 8, 9 or 11 (9: two passes for keys of up to 18 bits, the 1M scene's)
  int scorr_pow = 0;      // s_corr exponent shared by every s_corr scene (2-4), else 0
  // List entries per lane the list build stages in shared memory; a warp with
  // a longer list is finished by a second scan of its candidates.
  int stage_rows = kStageRowsDefault;
  // Some scene's clamped r^2 range, [(0.01 h)^2, h^2), lies outside the
  // range where the list passes' square root is checked against sqrtf (only
  // scenes whose kernel constants overflow or vanish): their passes use sqrtf.
  bool ieee_sqrt = false;
  // Per-kernel launch shape (indexed by FLUID_KERNEL_*), chosen by the
  // autotuner: neighbour entries fetched ahead (2, 4, 8; 1 when set
  // explicitly) in the list passes, and threads per block (128, 256, 512)
  // for the neighbour kernels.
  int unroll[FLUID_KERNEL_COUNT];
  int block[FLUID_KERNEL_COUNT];
  // Lanes per particle of the list passes (1, 2, 4, 8; see the several-lanes
  // kernels): above 1 the unroll is not used.
  int lanes[FLUID_KERNEL_COUNT];
  StepPlan() {
    for (int k = 0; k < FLUID_KERNEL_COUNT; ++k) {
      unroll[k] = 4;
      block[k] = kBlock;
      lanes[k] = 1;
    }
    // 128-thread blocks for the list passes: faster than 256 in the 1M lattice
    // step (0.974 -> 0.959 ms) and in collapsed states (125k: 8.17 -> 7.94 ms;
    // 1M step 22: 192.9 -> 187.8 ms) with four records ahead.
    for (int k : {FLUID_KERNEL_LAMBDA, FLUID_KERNEL_DELTA, FLUID_KERNEL_XSPH, FLUID_KERNEL_OMEGA, FLUID_KERNEL_ETA})
      block[k] = kDefaultListBlock;
  }
  // The default lanes per particle for a solver of `particles` in all. At
  // one lane a launch over a few thousand particles holds under a warp per
  // SM, so lambda and delta split each list over eight lanes there (four up
  // to 32,768); larger launches keep one, as the lanes' shuffles cost more
  // than they fill once the SMs have warps. Steps 1-20 from rest, ms per
  // step, one lane -> the default: dam breaks of 4,096 0.138 -> 0.094,
  // 15,625 1.45 -> 1.08, 21,952 2.88 -> 2.29, 32,768 5.35 -> 4.71 particles;
  // falling blocks of the same sizes 0.086 -> 0.080, 0.221 -> 0.173, 0.331 ->
  // 0.263, 0.508 -> 0.402. The 64,000-particle dam break (7k neighbours)
  // runs 13.1 ms at one lane and 16.7 at four.
  void size_for(long long particles) {
    const int g = particles <= kFewParticles ? 8 : particles <= kSomeParticles ? 4 : 1;
    lanes[FLUID_KERNEL_LAMBDA] = g;
    lanes[FLUID_KERNEL_DELTA] = g;
  }
};

// The s_corr exponent to compile into the delta pass: n when every scene with
// s_corr on uses the same n in {2, 3, 4}, else 0 (n read per scene).
inline int shared_scorr_pow(const SceneConst* sc, int scenes) {
  int n = 0;
  for (int s = 0; s < scenes; ++s) {
    if (!sc[s].scorr_on) continue;
    if (sc[s].scorr_n < 2 || sc[s].scorr_n > 4 || (n && n != sc[s].scorr_n)) return 0;
    n = sc[s].scorr_n;
  }
  return n;
}

// Kernels whose launch shape the autotuner chooses.
inline bool tunable_unroll(int k) {
  return k == FLUID_KERNEL_LAMBDA || k == FLUID_KERNEL_DELTA || k == FLUID_KERNEL_XSPH || k == FLUID_KERNEL_OMEGA ||
         k == FLUID_KERNEL_ETA;
}
inline bool tunable_block(int k) {
  return tunable_unroll(k) || k == FLUID_KERNEL_NBR_BUILD;
}

// Records an event after selected launches when profiling is on.
struct LaunchMarks {
  bool on = false;
  cudaStream_t stream = nullptr;
  bool capturing = false;
  std::vector<cudaEvent_t>* events = nullptr;  // events[0] recorded first
  std::vector<int>* stages = nullptr;          // stage of the launch ending at events[k]
  int next = 0;
  long long launches = 0;
  void start();
  void mark(int stage);
};

// Forward internals of one step kept for the adjoint (slot order of the
// step's output): x0 input positions, p = p^0..p^K (K+1 blocks of n),
// q = pre-projection positions of each iteration (K blocks), lambda (K
// blocks), rho of the last lambda pass.
struct StepRecord {
  float4* x0 = nullptr;
  float4* p = nullptr;
  float4* q = nullptr;
  float* lambda = nullptr;
  float* rho = nullptr;
  float4* omega = nullptr;  // omega and |omega| (when vorticity runs)
};

// The step's result written out while the step finishes (the stateless
// step on page-locked caller arrays): the positions, final once the last
// Jacobi iteration commits them, on `aux` while the velocity passes run; the
// velocities after the last pass. Both writes are skipped when the step
// failed, so a step that is re-run never exposes stale values.
// The six destination arrays (x, y, z positions, then velocities) are read
// from device memory, so a captured graph serves every call.
struct StepDownload {
  cudaStream_t aux = nullptr;
  cudaEvent_t committed = nullptr;       // recorded on the step's stream
  cudaEvent_t positions_done = nullptr;  // recorded on aux
  float* const* targets = nullptr;       // device array of 6 pointers
  // Blocks of the position write-out. The host link, not the SMs, bounds
  // it: a quarter of the SMs' worth of blocks keeps it at the link's rate
  // while leaving the rest to the velocity passes beside it (a full grid
  // slowed those passes by as much as the overlap saved).
  int blocks = 0;
  // The upload already added the predicted cells to the bounding box, so
  // the step starts at k_grid_setup.
  bool bounds_done = false;
};

// Enqueues one full timestep on `stream`; with `rec`, also records the
// internals the adjoint needs (device-to-device copies after the kernels);
// with `dl`, also writes the result out (see StepDownload).
cudaError_t enqueue_step(const StepArgs& a, const StepPlan& plan,
                         cudaStream_t stream, LaunchMarks& marks,
                         const StepRecord* rec = nullptr, const StepDownload* dl = nullptr);

// Packs caller-order SoA arrays (device) into slot-order x/v of one parity;
// with bmin/bmax it also accumulates the predicted cells' bounding box (what
// k_bounds does), for a step launched with StepDownload::bounds_done.
cudaError_t enqueue_upload(const float* px, const float* py, const float* pz,
                           const float* vx, const float* vy, const float* vz,
                           float4* x, float4* v, int* slot, float* rho,
                           const SceneConst* sc, int scenes, int n,
                           cudaStream_t stream, int* bmin = nullptr, int* bmax = nullptr);

// Gathers slot-order x/v of one parity into caller-order SoA arrays (device).
cudaError_t enqueue_download(const float4* x, const float4* v, const int* slot,
                             float* px, float* py, float* pz, float* vx,
                             float* vy, float* vz, int n, cudaStream_t stream);

// Resets the status word and the bounding-box accumulators.
cudaError_t enqueue_reset(DevStatus* status, int* bmin, int* bmax, int scenes,
                          cudaStream_t stream);

}  // namespace fgb
