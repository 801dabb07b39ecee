// Scene fills generated on the device, for scenes too large to fill on the
// host and copy over: the lattice block of core/src/init.cpp:72-106
// (init_block) with the seeded jitter the benchmark scenes add, and the cube
// and sphere shapes of a scene file (core/src/init.cpp:298-345). Each writes
// the caller's device SoA arrays in the reference's particle order, with the
// reference's float arithmetic, so a device fill equals the host fill bit for
// bit.
//
// The reference fills a shape with float loops `for (v = start; v < stop; v +=
// spacing)`: each coordinate is the previous one plus the spacing, rounded, so
// an axis is a sequential recurrence. The axes (at most a few thousand values
// each) are accumulated on the host exactly as the loops do; the device forms
// their product in the loops' order (x outermost, z innermost), and for a
// sphere keeps the points whose float (dx*dx + dy*dy) + dz*dz is below r*r, in
// order, by a per-block count, a scan of the block counts and a scatter.

#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "fluid_gb300.h"

namespace fgb {
namespace {

constexpr int kFillBlock = 256;
constexpr unsigned kFull = 0xffffffffu;

// SplitMix64 draw k (1-based) of `seed`: z = seed + k * golden, then the
// finaliser of Steele, Lea and Flood (2014).
__device__ __forceinline__ uint64_t splitmix64_at(uint64_t seed, uint64_t k) {
  uint64_t z = seed + k * 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// U(-a, a) rounded to float: a * (2u - 1) in double with u = (draw >> 11) *
// 2^-53, then rounded to nearest float (the host scenes' jitter, in numpy).
__device__ __forceinline__ float jitter_of(uint64_t seed, uint64_t k, double amplitude) {
  const double u = static_cast<double>(splitmix64_at(seed, k) >> 11) * (1.0 / 9007199254740992.0);
  return __double2float_rn(amplitude * (2.0 * u - 1.0));
}

// init_block (core/src/init.cpp:96-106): particle index = (z * ny + y) * nx
// + x at origin + float(i) * step per axis; then + jitter of draws 3m + 1,
// 3m + 2, 3m + 3 (m = first + particle index), added in float.
__global__ void __launch_bounds__(kFillBlock) k_fill_block(long long nx, long long ny, long long count, float ox,
                                                           float oy, float oz, float step, double amplitude,
                                                           uint64_t seed, long long first, float* px, float* py,
                                                           float* pz) {
  for (long long k = static_cast<long long>(blockIdx.x) * kFillBlock + threadIdx.x; k < count;
       k += static_cast<long long>(gridDim.x) * kFillBlock) {
    const long long x = k % nx;
    const long long y = (k / nx) % ny;
    const long long z = k / (nx * ny);
    float vx = __fadd_rn(ox, __fmul_rn(static_cast<float>(x), step));
    float vy = __fadd_rn(oy, __fmul_rn(static_cast<float>(y), step));
    float vz = __fadd_rn(oz, __fmul_rn(static_cast<float>(z), step));
    if (amplitude != 0.0) {
      const uint64_t d = 3ull * static_cast<uint64_t>(first + k);
      vx = __fadd_rn(vx, jitter_of(seed, d + 1, amplitude));
      vy = __fadd_rn(vy, jitter_of(seed, d + 2, amplitude));
      vz = __fadd_rn(vz, jitter_of(seed, d + 3, amplitude));
    }
    px[k] = vx;
    py[k] = vy;
    pz[k] = vz;
  }
}

struct Axes {
  const float* v[3];
  long long n[3];
};

// Lattice point k of the three axes in loop order (x outermost, z innermost).
__device__ __forceinline__ void point_of(const Axes& ax, long long k, float& x, float& y, float& z) {
  const long long iz = k % ax.n[2];
  const long long iy = (k / ax.n[2]) % ax.n[1];
  const long long ix = k / (ax.n[2] * ax.n[1]);
  x = ax.v[0][ix];
  y = ax.v[1][iy];
  z = ax.v[2][iz];
}

// Sphere membership (core/src/init.cpp:336-339): (dx*dx + dy*dy) + dz*dz < r2,
// each operation rounded.
__device__ __forceinline__ bool in_sphere(float x, float y, float z, float cx, float cy, float cz, float r2) {
  const float dx = __fsub_rn(x, cx), dy = __fsub_rn(y, cy), dz = __fsub_rn(z, cz);
  return __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)) < r2;
}

// Kept points per block of kFillBlock lattice points (sphere = 0: all).
__global__ void __launch_bounds__(kFillBlock) k_shape_count(Axes ax, long long total, int sphere, float cx, float cy,
                                                            float cz, float r2, int* block_count) {
  const long long k = static_cast<long long>(blockIdx.x) * kFillBlock + threadIdx.x;
  bool keep = false;
  if (k < total) {
    float x, y, z;
    point_of(ax, k, x, y, z);
    keep = !sphere || in_sphere(x, y, z, cx, cy, cz, r2);
  }
  const int c = __popc(__ballot_sync(kFull, keep));
  __shared__ int warp_count[kFillBlock / 32];
  if ((threadIdx.x & 31) == 0) warp_count[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    int s = 0;
    for (int w = 0; w < kFillBlock / 32; ++w) s += warp_count[w];
    block_count[blockIdx.x] = s;
  }
}

// Exclusive scan of the block counts, one block; writes the total last.
__global__ void __launch_bounds__(1024) k_shape_scan(int* block_count, int blocks) {
  __shared__ int carry;
  __shared__ int warp_sum[32];
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < blocks; base += 1024) {
    const int b = base + threadIdx.x;
    const int v = b < blocks ? block_count[b] : 0;
    int inc = v;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(kFull, inc, o);
      if (lane >= o) inc += y;
    }
    if (lane == 31) warp_sum[warp] = inc;
    __syncthreads();
    int before = carry;
    for (int w = 0; w < warp; ++w) before += warp_sum[w];
    if (b < blocks) block_count[b] = before + inc - v;
    __syncthreads();
    if (threadIdx.x == 1023) carry = before + inc;
    __syncthreads();
  }
  if (threadIdx.x == 0) block_count[blocks] = carry;
}

// Kept points in order: block offset + rank inside the block.
__global__ void __launch_bounds__(kFillBlock) k_shape_write(Axes ax, long long total, int sphere, float cx, float cy,
                                                            float cz, float r2, const int* block_start, float vx,
                                                            float vy, float vz, float* px, float* py, float* pz,
                                                            float* ux, float* uy, float* uz) {
  const long long k = static_cast<long long>(blockIdx.x) * kFillBlock + threadIdx.x;
  float x = 0.0f, y = 0.0f, z = 0.0f;
  bool keep = false;
  if (k < total) {
    point_of(ax, k, x, y, z);
    keep = !sphere || in_sphere(x, y, z, cx, cy, cz, r2);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned b = __ballot_sync(kFull, keep);
  __shared__ int warp_count[kFillBlock / 32];
  if (lane == 0) warp_count[warp] = __popc(b);
  __syncthreads();
  if (!keep) return;
  int o = block_start[blockIdx.x] + __popc(b & ((1u << lane) - 1u));
  for (int w = 0; w < warp; ++w) o += warp_count[w];
  px[o] = x;
  py[o] = y;
  pz[o] = z;
  ux[o] = vx;
  uy[o] = vy;
  uz[o] = vz;
}

// One axis of a shape: for (v = start; v < stop; v += step) in float. False
// when the loop would not end in 2^24 values (a spacing below the
// coordinates' ulp never advances; the reference's loop would not end).
bool fill_axis(float start, float stop, float step, std::vector<float>& out) {
  out.clear();
  for (float v = start; v < stop; v += step) {
    if (out.size() >= (1u << 24)) return false;
    out.push_back(v);
  }
  return true;
}

}  // namespace
}  // namespace fgb

extern "C" int fluid_fill_block(int64_t nx, int64_t ny, int64_t nz, float origin_x, float origin_y, float origin_z,
                                float spacing, double jitter, uint64_t seed, int64_t first, float* pos_x,
                                float* pos_y, float* pos_z, void* stream) {
  using namespace fgb;
  if (nx < 0 || ny < 0 || nz < 0 || !(spacing > 0.0f) || !(jitter >= 0.0) || first < 0)
    return FLUID_ERR_INVALID_ARGUMENT;
  const long long count = nx * ny * nz;
  if (count == 0) return FLUID_OK;
  if (!pos_x || !pos_y || !pos_z) return FLUID_ERR_INVALID_ARGUMENT;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const long long want = (count + kFillBlock - 1) / kFillBlock;
  const int blocks = static_cast<int>(want < 65536 ? want : 65536);
  k_fill_block<<<blocks, kFillBlock, 0, st>>>(nx, ny, count, origin_x, origin_y, origin_z, spacing, jitter, seed,
                                              first, pos_x, pos_y, pos_z);
  if (cudaGetLastError() != cudaSuccess) return FLUID_ERR_CUDA;
  return cudaStreamSynchronize(st) == cudaSuccess ? FLUID_OK : FLUID_ERR_CUDA;
}

extern "C" int fluid_fill_shape(int32_t kind, const float origin[3], const float extent[3], float spacing,
                                const float velocity[3], float* pos_x, float* pos_y, float* pos_z, float* vel_x,
                                float* vel_y, float* vel_z, int64_t capacity, int64_t* count, void* stream) {
  using namespace fgb;
  if (!origin || !extent || !count || (kind != FLUID_SHAPE_CUBE && kind != FLUID_SHAPE_SPHERE) ||
      !(spacing > 0.0f) || capacity < 0)
    return FLUID_ERR_INVALID_ARGUMENT;
  *count = 0;
  const bool sphere = kind == FLUID_SHAPE_SPHERE;
  const float half = spacing * 0.5f;
  std::vector<float> axis[3];
  for (int d = 0; d < 3; ++d) {
    const bool ok = sphere ? fill_axis(origin[d] - extent[0] + half, origin[d] + extent[0], spacing, axis[d])  // :329-334
                           : fill_axis(origin[d] + half, origin[d] + extent[d], spacing, axis[d]);           // :298-300
    if (!ok) return FLUID_ERR_INVALID_ARGUMENT;
  }
  const long long total = static_cast<long long>(axis[0].size()) * axis[1].size() * axis[2].size();
  if (total == 0) return FLUID_OK;
  if (total > (1ll << 31) - 1) return FLUID_ERR_INVALID_ARGUMENT;
  const float r2 = sphere ? extent[0] * extent[0] : 0.0f;
  const float vx = velocity ? velocity[0] : 0.0f, vy = velocity ? velocity[1] : 0.0f, vz = velocity ? velocity[2] : 0.0f;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int blocks = static_cast<int>((total + kFillBlock - 1) / kFillBlock);
  // One device allocation for this call: the three axes and the block counts.
  const size_t axis_bytes = sizeof(float) * (axis[0].size() + axis[1].size() + axis[2].size());
  const size_t bytes = axis_bytes + sizeof(int) * (static_cast<size_t>(blocks) + 1);
  void* scratch = nullptr;
  if (cudaMalloc(&scratch, bytes) != cudaSuccess) return FLUID_ERR_OUT_OF_MEMORY;
  float* dax = static_cast<float*>(scratch);
  int* block_count = reinterpret_cast<int*>(static_cast<char*>(scratch) + axis_bytes);
  std::vector<float> packed;
  packed.reserve(axis_bytes / sizeof(float));
  for (int d = 0; d < 3; ++d) packed.insert(packed.end(), axis[d].begin(), axis[d].end());
  Axes ax;
  ax.v[0] = dax;
  ax.v[1] = dax + axis[0].size();
  ax.v[2] = dax + axis[0].size() + axis[1].size();
  for (int d = 0; d < 3; ++d) ax.n[d] = static_cast<long long>(axis[d].size());
  int rc = FLUID_OK;
  int kept = 0;
  if (cudaMemcpyAsync(dax, packed.data(), axis_bytes, cudaMemcpyHostToDevice, st) != cudaSuccess) rc = FLUID_ERR_CUDA;
  if (!rc) {
    k_shape_count<<<blocks, kFillBlock, 0, st>>>(ax, total, sphere, origin[0], origin[1], origin[2], r2, block_count);
    k_shape_scan<<<1, 1024, 0, st>>>(block_count, blocks);
    if (cudaGetLastError() != cudaSuccess ||
        cudaMemcpyAsync(&kept, block_count + blocks, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
      rc = FLUID_ERR_CUDA;
  }
  if (!rc) {
    *count = kept;
    if (kept > capacity) {
      rc = FLUID_ERR_CAPACITY;  // *count tells the caller how much to allocate
    } else if (kept > 0) {
      if (!pos_x || !pos_y || !pos_z || !vel_x || !vel_y || !vel_z) {
        rc = FLUID_ERR_INVALID_ARGUMENT;
      } else {
        k_shape_write<<<blocks, kFillBlock, 0, st>>>(ax, total, sphere, origin[0], origin[1], origin[2], r2,
                                                     block_count, vx, vy, vz, pos_x, pos_y, pos_z, vel_x, vel_y,
                                                     vel_z);
        if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(st) != cudaSuccess) rc = FLUID_ERR_CUDA;
      }
    }
  }
  cudaStreamSynchronize(st);
  cudaFree(scratch);
  return rc;
}
