// One PBF timestep that allocates nothing: fluid_gb300_step_noalloc.
//
// Some callers cannot allocate device memory at the point where they step
// the fluid: a host application or engine that owns every device allocation
// through its own pool or budget, code running where an allocation would
// stall or synchronise the device in a frame-time or real-time loop, or a
// plugin that must not grow the process's footprint behind the host's back.
// For them this entry point runs the same kernels as every other step, but all
// of its scratch (sorted state, sort buffers, cell table, neighbour lists,
// status word) lives in one fixed, file-scope device array sized for
// FLUID_NOALLOC_MAX_PARTICLES particles. Inputs and outputs stay the caller's
// own device arrays.
//
// The array belongs to every GPU that loads this library, for the life of the
// process. All calls share it and it keeps the last call's contents, so calls
// whose work overlaps on the GPU (two streams, two threads, two devices'
// worth of calls aimed at one device) race on it; serialise them. What must
// start at zero (the status word and the bounding-box accumulators) is reset
// by every call; the cell table needs no clearing (its entries are validated).

#include <cuda_runtime.h>

#include <mutex>

#include "fluid_gb300.h"
#include "pbf_common.cuh"
#include "pbf_launch.h"

namespace fgb {

SceneConst scene_const_for(const fluid_params& p, int first, int count);
int params_status(const fluid_params& p);

namespace {

constexpr size_t kAlign = 256;
constexpr size_t up(size_t v) { return (v + kAlign - 1) / kAlign * kAlign; }

constexpr int kMaxN = FLUID_NOALLOC_MAX_PARTICLES;
constexpr long long kMaxSlots = FLUID_NOALLOC_MAX_NEIGHBOR_SLOTS;
constexpr long long kMaxCells = FLUID_NOALLOC_MAX_CELLS;
constexpr int kMaxWarps = kMaxN / 32;
constexpr int kMaxTiles = (kMaxN + kRadixTile - 1) / kRadixTile;

constexpr size_t kF4 = up(sizeof(float4) * kMaxN);
constexpr size_t kI32 = up(sizeof(int) * kMaxN);

// Byte offsets of every buffer inside the arena.
constexpr size_t kX0 = 0, kX1 = kX0 + kF4, kV0 = kX1 + kF4, kV1 = kV0 + kF4;
constexpr size_t kP0 = kV1 + kF4, kP1 = kP0 + kF4, kV2 = kP1 + kF4, kOmega = kV2 + kF4;
constexpr size_t kPl = kOmega + kF4;
constexpr size_t kLive = kPl + kF4;
constexpr size_t kSlot0 = kLive + up(2 * sizeof(uint32_t) * kMaxN), kSlot1 = kSlot0 + kI32, kRho0 = kSlot1 + kI32, kRho1 = kRho0 + kI32;
constexpr size_t kLambda = kRho1 + kI32, kKeys0 = kLambda + kI32, kKeys1 = kKeys0 + kI32;
constexpr size_t kVals0 = kKeys1 + kI32, kVals1 = kVals0 + kI32, kCnt = kVals1 + kI32;
constexpr size_t kDepth = kCnt + kI32, kWbase = kDepth + up(sizeof(int) * (kMaxWarps + 1));
constexpr size_t kOvf = kWbase + up(sizeof(long long) * (kMaxWarps + 1));
constexpr size_t kLook = kOvf + up(sizeof(int) * (kMaxWarps + 1));
constexpr size_t kRadixNext = kLook + up(sizeof(unsigned long long) * kRadixMaxBins * kMaxTiles);
constexpr size_t kDigits = kRadixNext + up(sizeof(int) * kRadixMaxPasses);
constexpr size_t kBmin = kDigits + up(sizeof(uint32_t) * kRadixMaxBins * kRadixMaxPasses);
constexpr size_t kBmax = kBmin + up(3 * sizeof(int));
constexpr size_t kGrid = kBmax + up(3 * sizeof(int));
constexpr size_t kStatus = kGrid + up(sizeof(GridInfo));
constexpr size_t kConst = kStatus + up(sizeof(DevStatus));
constexpr size_t kTable = kConst + up(sizeof(SceneConst));
constexpr size_t kNbr = kTable + up(sizeof(int2) * kMaxCells);
constexpr size_t kScratchBytes = kNbr + up(sizeof(int) * kMaxSlots);
static_assert(kScratchBytes < (8u << 20), "the no-allocation arena should stay under 8 MiB");

// The scratch arena: the only device memory this entry point uses besides the
// caller's arrays.
static __device__ __align__(256) unsigned char g_step_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
unsigned char* g_base[kMaxDevices] = {};

// Device address of the arena on the current device. Host code cannot use
// g_step_scratch directly (in host code it names a host-side stand-in), so
// the address is looked up once per device, with that device current.
unsigned char* arena_for(int device) {
  if (device < 0 || device >= kMaxDevices) return nullptr;
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_base[device]) {
    void* ptr = nullptr;
    if (cudaGetSymbolAddress(&ptr, g_step_scratch) != cudaSuccess || !ptr) return nullptr;
    g_base[device] = static_cast<unsigned char*>(ptr);
  }
  return g_base[device];
}

template <typename T>
T* at(unsigned char* base, size_t off) {
  return reinterpret_cast<T*>(base + off);
}

StepArgs carve(unsigned char* b, int n) {
  StepArgs a{};
  a.x_old = at<float4>(b, kX0);
  a.v_old = at<float4>(b, kV0);
  a.slot_old = at<int>(b, kSlot0);
  a.rho_old = at<float>(b, kRho0);
  a.x = at<float4>(b, kX1);
  a.v = at<float4>(b, kV1);
  a.v2 = at<float4>(b, kV2);
  a.slot = at<int>(b, kSlot1);
  a.p[0] = at<float4>(b, kP0);
  a.p[1] = at<float4>(b, kP1);
  a.omega = at<float4>(b, kOmega);
  a.pl = at<float4>(b, kPl);
  a.live = at<uint32_t>(b, kLive);
  a.lambda = at<float>(b, kLambda);
  a.rho = at<float>(b, kRho1);
  a.keys[0] = at<uint32_t>(b, kKeys0);
  a.keys[1] = at<uint32_t>(b, kKeys1);
  a.vals[0] = at<int>(b, kVals0);
  a.vals[1] = at<int>(b, kVals1);
  a.look = at<unsigned long long>(b, kLook);
  a.radix_next = at<int>(b, kRadixNext);
  a.digit_total = at<uint32_t>(b, kDigits);
  a.table = at<int2>(b, kTable);
  a.cnt = at<int>(b, kCnt);
  a.depth = at<int>(b, kDepth);
  a.wbase = at<long long>(b, kWbase);
  a.slice_fmt = at<int>(b, kOvf);
  a.list16 = 1;
  a.nbr = at<int>(b, kNbr);
  a.bmin = at<int>(b, kBmin);
  a.bmax = at<int>(b, kBmax);
  a.grid = at<GridInfo>(b, kGrid);
  a.status = at<DevStatus>(b, kStatus);
  a.sc = at<SceneConst>(b, kConst);
  a.n = n;
  a.scenes = 1;
  a.tiles = (n + kRadixTile - 1) / kRadixTile;
  a.warps = (n + 31) / 32;
  a.grid_capacity = kMaxCells;
  a.nbr_capacity = kMaxSlots;
  return a;
}

}  // namespace
}  // namespace fgb

extern "C" int fluid_gb300_step_noalloc(const fluid_params* params, int64_t count, float* pos_x, float* pos_y,
                                        float* pos_z, float* vel_x, float* vel_y, float* vel_z, float* time,
                                        void* stream) {
  using namespace fgb;
  if (!params || !time || count < 0) return FLUID_ERR_INVALID_ARGUMENT;
  if (count > kMaxN) return FLUID_ERR_CAPACITY;
  const int prc = params_status(*params);
  if (prc) return prc;
  if (count == 0) {
    *time += params->dt;
    return FLUID_OK;
  }
  if (!pos_x || !pos_y || !pos_z || !vel_x || !vel_y || !vel_z) return FLUID_ERR_INVALID_ARGUMENT;
  int device = -1;
  if (cudaGetDevice(&device) != cudaSuccess) return FLUID_ERR_NO_DEVICE;
  unsigned char* base = arena_for(device);
  if (!base) return FLUID_ERR_CUDA;

  const int n = static_cast<int>(count);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  StepArgs a = carve(base, n);
  const SceneConst c = scene_const_for(*params, 0, n);
  StepPlan plan;
  plan.size_for(n);
  plan.iterations = c.iterations;
  plan.xsph = c.xsph_on != 0;
  plan.vorticity = c.vort_on != 0;
  plan.restitution = c.rest_on != 0;
  plan.radix_bits = 8;
  plan.radix_passes = 3;  // keys < FLUID_NOALLOC_MAX_CELLS = 2^18
  plan.scorr_pow = shared_scorr_pow(&c, 1);
  plan.ieee_sqrt = c.exact_sqrt != 0;
  LaunchMarks marks;      // profiling off

  if (cudaMemcpyAsync(const_cast<SceneConst*>(a.sc), &c, sizeof(c), cudaMemcpyHostToDevice, st) != cudaSuccess)
    return FLUID_ERR_CUDA;
  if (enqueue_reset(a.status, a.bmin, a.bmax, 1, st) != cudaSuccess) return FLUID_ERR_CUDA;
  if (enqueue_upload(pos_x, pos_y, pos_z, vel_x, vel_y, vel_z, const_cast<float4*>(a.x_old),
                     const_cast<float4*>(a.v_old), const_cast<int*>(a.slot_old), const_cast<float*>(a.rho_old),
                     a.sc, 1, n, st) != cudaSuccess)
    return FLUID_ERR_CUDA;
  if (enqueue_step(a, plan, st, marks) != cudaSuccess) return FLUID_ERR_CUDA;
  // The status word is read on the caller's stream, behind the step, so the
  // call waits on that stream only (not on other streams of the device).
  DevStatus status;
  if (cudaMemcpyAsync(&status, a.status, sizeof(status), cudaMemcpyDeviceToHost, st) != cudaSuccess)
    return FLUID_ERR_CUDA;
  if (cudaStreamSynchronize(st) != cudaSuccess) return FLUID_ERR_CUDA;
  if (status.err) return status.err;  // caller's arrays untouched
  if (enqueue_download(a.x, a.v, a.slot, pos_x, pos_y, pos_z, vel_x, vel_y, vel_z, n, st) != cudaSuccess)
    return FLUID_ERR_CUDA;
  if (cudaStreamSynchronize(st) != cudaSuccess) return FLUID_ERR_CUDA;
  *time += params->dt;
  return FLUID_OK;
}
