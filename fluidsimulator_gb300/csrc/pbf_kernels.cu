// GB300 (sm_103a) kernels of the Position Based Fluids timestep.
//
// One timestep, in launch order (reference: core/src/core.cpp:119-615):
//   k_bounds        predicted cell of every particle, per-scene bounding box
//   k_grid_setup    per-scene dense grid over that box, key base, radix passes
//   k_keys          x-major linear cell key per particle, in caller order
//   k_radix_digits  digit counts of every sort pass, one read of the keys
//   k_radix_onesweep  one stable LSD pass of (key, caller index), 8-, 9- or 11-bit
//                   digits: tile ranking, decoupled look-back, scatter
//   k_reorder       gather into cell order, predict again (bit-identical),
//                   cell (first, end) table by warp-shuffle boundary detection
//   k_nbr_build     27-cell scan: lists in scan order staged in shared memory,
//                   slices claimed by one atomic per block, coalesced copy-out;
//                   capacity check; a second scan for warps whose lists
//                   outgrew the staging
//   k_lambda        density / lambda (iterations 1-3 also record which of
//                   each list's first 64 entries are within h: live bits)
//   k_delta         position correction, s_corr, plane projection (last
//                   iteration also commits v = (p - x)/dt, x = p); iterations
//                   1-3 walk only the live ones of those entries
//   k_xsph          XSPH viscosity over the step's lists (records live bits
//                   at the committed positions)
//   k_omega, k_eta  vorticity confinement (+ plane restitution / friction),
//                   walking only the live ones of the first 64 entries
//
// Arithmetic follows the reference's float operations one for one: the
// library is compiled with -fmad=false (no contraction), IEEE division and
// square root, and each neighbour sum runs in the reference's order (cells
// dz, dy, dx; ascending caller index inside a cell), so on the same input the
// results equal the reference CPU path bit for bit. Membership tests and the
// prediction use explicit round-to-nearest intrinsics as well; the list
// passes form each neighbour's terms two at a time in paired FP32
// instructions whose lanes round as the scalar operations do (see pmul).

#include <climits>
#include <type_traits>
#include <cstdint>

#include "pbf_common.cuh"
#include "pbf_launch.h"

namespace fgb {
namespace {

constexpr int kMaxBlock = 512;  // largest block the tuner may pick
// Minimum resident 512-thread blocks the list passes are compiled for (caps
// their registers: 1 -> 128, 2 -> 64, 3 -> 42 per thread).
#ifndef FGB_LIST_MIN_BLOCKS
#define FGB_LIST_MIN_BLOCKS 2
#endif
constexpr int kMaxBuildBlock = kMaxStageBlock;  // k_nbr_build: stage_rows + 1 ints per thread of shared memory
// List entries per lane staged in shared memory by the list build: the step
// plan's stage_rows (+ a spare row), kStageRowsDefault = 36 unless a step's
// lists were longer and fit kMaxStageRows (37 KB per 256-thread block at 36).
// Lattice-phase lists hold at most ~32 entries; every staged row is shared
// memory the L1 cannot use for the candidates the scan reads (5 blocks per
// SM), so the build ran 0.295 ms at 40 and 0.284 ms at 36 or 32 per 1M step.
// A warp with longer lists scans its candidates a second time.

__device__ __forceinline__ bool failed(const DevStatus* st) {
  return *reinterpret_cast<const volatile int*>(&st->err) != 0;
}

__device__ __forceinline__ void set_error(DevStatus* st, int code) {
  if (atomicCAS(&st->err, 0, code) == 0) st->fail_step = st->step;
}

__device__ __forceinline__ unsigned lanemask_lt(int lane) { return (1u << lane) - 1u; }

// v += f dt; p = x + v dt  (core.cpp:154-160), each operation rounded.
__device__ __forceinline__ float4 predict(const SceneConst& c, const float4 x, float4& v) {
  v.x = __fadd_rn(v.x, c.gdt_x);
  v.y = __fadd_rn(v.y, c.gdt_y);
  v.z = __fadd_rn(v.z, c.gdt_z);
  float4 p;
  p.x = __fadd_rn(x.x, __fmul_rn(v.x, c.dt));
  p.y = __fadd_rn(x.y, __fmul_rn(v.y, c.dt));
  p.z = __fadd_rn(x.z, __fmul_rn(v.z, c.dt));
  p.w = v.w;
  return p;
}

// floor(p * (1/h)) per axis (core.cpp:28-34). False when out of range / NaN.
__device__ __forceinline__ bool cell_of(const SceneConst& c, const float4 p, int& cx, int& cy, int& cz) {
  const float fx = __fmul_rn(p.x, c.inv_h);
  const float fy = __fmul_rn(p.y, c.inv_h);
  const float fz = __fmul_rn(p.z, c.inv_h);
  if (!(fabsf(fx) < 1.0e9f && fabsf(fy) < 1.0e9f && fabsf(fz) < 1.0e9f)) return false;
  cx = static_cast<int>(floorf(fx));
  cy = static_cast<int>(floorf(fy));
  cz = static_cast<int>(floorf(fz));
  return true;
}

// (dx*dx + dy*dy) + dz*dz, each operation rounded (core.cpp:234-237).
__device__ __forceinline__ float dist2(float dx, float dy, float dz) {
  return __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
}

// Paired FP32 arithmetic: two IEEE round-to-nearest operations per
// instruction (sm_100 and later); each half equals the scalar operation.
__device__ __forceinline__ float2 f2(float v) { return make_float2(v, v); }
__device__ __forceinline__ float2 padd(float2 a, float2 b) { return __fadd2_rn(a, b); }
// a * b rounded once, written as fma(a, b, nz) with nz = -0.0 read from
// memory (SceneConst::neg_zero). A paired multiply whose result feeds a
// paired add is contracted into one fused multiply-add by the code generator
// even with explicit round-to-nearest and contraction disabled (measured: the
// sum then equals fma(x, x, y * y)), which rounds once where the reference
// rounds twice. An fma with an addend unknown at compile time cannot be
// contracted further, and RN(a * b + (-0)) = RN(a * b) for every a and b,
// signed zeros included.
__device__ __forceinline__ float2 pmul(float2 a, float2 b, float2 nz) { return __ffma2_rn(a, b, nz); }
// a - b rounded once, as fma(b, -1, a): b * -1 is exact, and the signs of
// zero come out as in a - b. No operand of a psub comes from a pmul.
__device__ __forceinline__ float2 psub(float2 a, float2 b) { return __ffma2_rn(b, f2(-1.0f), a); }

// W_poly6 for r2 < h2 (core.cpp:35-46): coeff * ((d*d)*d), d = h2 - r2.
__device__ __forceinline__ float poly6(const SceneConst& c, float r2) {
  const float d = c.h2 - r2;
  return c.poly6_c * (d * d * d);
}

// Spiky gradient factor (core.cpp:48-57): (coeff * (h - r)) * (h - r).
__device__ __forceinline__ float spiky(const SceneConst& c, float r) {
  if (r > c.h) return 0.0f;
  const float d = c.h - r;
  return c.spiky_c * d * d;
}

// r from r^2 with the 0.01 h floor (core.cpp:303), correctly rounded:
// rn_sqrt (checked over every scene's clamped r^2 range unless the step's
// plan says otherwise), or sqrtf in the kIeee instantiations and the
// vorticity pass.
template <bool kIeee = false>
__device__ __forceinline__ float clamped_r(const SceneConst& c, float r2) {
  const float x = r2 < c.min_r2 ? c.min_r2 : r2;
  return kIeee ? sqrtf(x) : rn_sqrt(x);
}

// ratio^n (core.cpp:59-71).
__device__ __forceinline__ float pow_n(float r, int n) {
  if (n == 2) return r * r;
  if (n == 3) return r * r * r;
  if (n == 4) {
    const float r2 = r * r;
    return r2 * r2;
  }
  return powf(r, static_cast<float>(n));
}

// ratio^n with n fixed at compile time (kPow 2, 3 or 4), or read per scene
// (kPow 0); the same operations as pow_n.
template <int kPow>
__device__ __forceinline__ float pow_k(float r, int n) {
  if (kPow == 2) return r * r;
  if (kPow == 3) return r * r * r;
  if (kPow == 4) {
    const float r2 = r * r;
    return r2 * r2;
  }
  return pow_n(r, n);
}

// Paired forms of the per-entry geometry and kernel functions, for two list
// entries a and b at once; every lane rounds exactly as the scalar form.
// d = p - q per axis and r2 = dist2(d).
struct PairGeom {
  float2 dx, dy, dz, r2;
};
__device__ __forceinline__ PairGeom pair_geom(const float2 px, const float2 py, const float2 pz, const float4 qa,
                                              const float4 qb, const float2 nz) {
  PairGeom g;
  g.dx = psub(px, make_float2(qa.x, qb.x));
  g.dy = psub(py, make_float2(qa.y, qb.y));
  g.dz = psub(pz, make_float2(qa.z, qb.z));
  g.r2 = padd(padd(pmul(g.dx, g.dx, nz), pmul(g.dy, g.dy, nz)), pmul(g.dz, g.dz, nz));
  return g;
}
// poly6 of both lanes.
__device__ __forceinline__ float2 poly6_pair(const SceneConst& c, const float2 r2, const float2 nz) {
  const float2 d = psub(f2(c.h2), r2);
  return pmul(f2(c.poly6_c), pmul(pmul(d, d, nz), d, nz), nz);
}
// spiky(clamped_r(r2)) of both lanes.
template <bool kIeee = false>
__device__ __forceinline__ float2 spiky_pair(const SceneConst& c, const float2 r2, const float2 nz) {
  const float2 x = make_float2(r2.x < c.min_r2 ? c.min_r2 : r2.x, r2.y < c.min_r2 ? c.min_r2 : r2.y);
  const float2 r = kIeee ? make_float2(sqrtf(x.x), sqrtf(x.y)) : rn_sqrt2(x, nz);
  const float2 e = psub(f2(c.h), r);
  float2 gf = pmul(pmul(f2(c.spiky_c), e, nz), e, nz);
  if (r.x > c.h) gf.x = 0.0f;
  if (r.y > c.h) gf.y = 0.0f;
  return gf;
}

// Plane restitution and friction on velocity (core.cpp:586-606); each plane
// has its own tangential scale 1 - friction.
__device__ __forceinline__ void restitution(const SceneConst& c, float px, float py, float pz,
                                            float& vx, float& vy, float& vz) {
  for (int q = 0; q < c.plane_count; ++q) {
    const float4 pl = c.planes[q];
    const float sd = pl.x * px + pl.y * py + pl.z * pz - pl.w;
    if (sd <= 0.0f) {
      const float vn = pl.x * vx + pl.y * vy + pl.z * vz;
      float vn_new = vn;
      if (vn < 0.0f) vn_new = c.rest_neg_e * vn;
      const float tx = vx - vn * pl.x;
      const float ty = vy - vn * pl.y;
      const float tz = vz - vn * pl.z;
      const float keep = c.rest_scale[q];
      vx = tx * keep + vn_new * pl.x;
      vy = ty * keep + vn_new * pl.y;
      vz = tz * keep + vn_new * pl.z;
    }
  }
}

__device__ __forceinline__ const uint32_t* sorted_keys(const StepArgs& a, int npass) {
  return a.keys[npass & 1];
}

__device__ __forceinline__ uint32_t cell_key(const GridInfo& g, int cx, int cy, int cz) {
  const long long l = (static_cast<long long>(cx - g.minx) * g.dimy + (cy - g.miny)) * g.dimz + (cz - g.minz);
  return g.base + static_cast<uint32_t>(l);
}

// ---------------------------------------------------------------------------
// Bounds, grid, keys

// Adds each thread's predicted cell (ok) of `scene` (< 0: none) to the
// per-scene bounding box: warp, then block reduction when the block is one
// scene; mixed blocks (scene boundaries) fall back to per-warp or per-lane
// atomics. Called by every thread of a kBlock-thread block.
__device__ __forceinline__ void add_bounds(int* bmin, int* bmax, int scene, bool ok, int cx, int cy, int cz) {
  __shared__ int wmin[kBlock / 32][3], wmax[kBlock / 32][3], wscene[kBlock / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int s0 = __shfl_sync(kFull, scene, 0);
  const bool uniform = __all_sync(kFull, scene == s0 || scene < 0);
  int mn[3] = {INT_MAX, INT_MAX, INT_MAX}, mx[3] = {INT_MIN, INT_MIN, INT_MIN};
  if (uniform) {
    mn[0] = __reduce_min_sync(kFull, ok ? cx : INT_MAX);
    mn[1] = __reduce_min_sync(kFull, ok ? cy : INT_MAX);
    mn[2] = __reduce_min_sync(kFull, ok ? cz : INT_MAX);
    mx[0] = __reduce_max_sync(kFull, ok ? cx : INT_MIN);
    mx[1] = __reduce_max_sync(kFull, ok ? cy : INT_MIN);
    mx[2] = __reduce_max_sync(kFull, ok ? cz : INT_MIN);
  } else if (ok) {
    atomicMin(&bmin[3 * scene + 0], cx);
    atomicMin(&bmin[3 * scene + 1], cy);
    atomicMin(&bmin[3 * scene + 2], cz);
    atomicMax(&bmax[3 * scene + 0], cx);
    atomicMax(&bmax[3 * scene + 1], cy);
    atomicMax(&bmax[3 * scene + 2], cz);
  }
  if (lane == 0) {
    wscene[warp] = (uniform && mn[0] != INT_MAX) ? s0 : -1;
    for (int d = 0; d < 3; ++d) {
      wmin[warp][d] = mn[d];
      wmax[warp][d] = mx[d];
    }
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  int bs = -1;
  bool same = true;
  for (int w = 0; w < kBlock / 32; ++w) {
    if (wscene[w] < 0) continue;
    if (bs < 0) bs = wscene[w];
    else if (wscene[w] != bs) same = false;
  }
  if (bs < 0) return;
  if (same) {
    for (int d = 0; d < 3; ++d) {
      int lo = INT_MAX, hi = INT_MIN;
      for (int w = 0; w < kBlock / 32; ++w) {
        if (wscene[w] < 0) continue;
        lo = min(lo, wmin[w][d]);
        hi = max(hi, wmax[w][d]);
      }
      atomicMin(&bmin[3 * bs + d], lo);
      atomicMax(&bmax[3 * bs + d], hi);
    }
  } else {
    for (int w = 0; w < kBlock / 32; ++w) {
      if (wscene[w] < 0) continue;
      for (int d = 0; d < 3; ++d) {
        atomicMin(&bmin[3 * wscene[w] + d], wmin[w][d]);
        atomicMax(&bmax[3 * wscene[w] + d], wmax[w][d]);
      }
    }
  }
}

__global__ void __launch_bounds__(kBlock) k_bounds(StepArgs a) {
  if (failed(a.status)) return;
  const int s = blockIdx.x * kBlock + threadIdx.x;
  int scene = -1;
  int cx = 0, cy = 0, cz = 0;
  bool ok = false;
  if (s < a.n) {
    const float4 x = a.x_old[s];
    float4 v = a.v_old[s];
    scene = __float_as_int(v.w);
    const SceneConst& c = a.sc[scene];
    ok = cell_of(c, predict(c, x, v), cx, cy, cz);
  }
  add_bounds(a.bmin, a.bmax, scene, ok, cx, cy, cz);
}

// radix_bits: digit width of the sort (8, 9 or 11), which sets the pass count.
__global__ void __launch_bounds__(kBlock) k_grid_setup(StepArgs a, int radix_bits) {
  if (failed(a.status)) return;
  DevStatus* st = a.status;
  for (int i = threadIdx.x; i < kRadixMaxPasses * kRadixMaxBins; i += blockDim.x) a.digit_total[i] = 0;
  if (threadIdx.x < kRadixMaxPasses) a.radix_next[threadIdx.x] = 0;
  if (threadIdx.x != 0) return;
  st->epoch = st->epoch + 1u;  // look-back words of earlier steps no longer match
  st->step = st->started;
  st->started = st->started + 1;
  st->pairs = 0ull;
  st->cursor = 0ull;
  st->nbr_max = 0;
  unsigned long long total = 0;
  bool domain = false;
  for (int s = 0; s < a.scenes; ++s) {
    GridInfo g;
    g.minx = a.bmin[3 * s + 0];
    g.miny = a.bmin[3 * s + 1];
    g.minz = a.bmin[3 * s + 2];
    const int mxx = a.bmax[3 * s + 0], mxy = a.bmax[3 * s + 1], mxz = a.bmax[3 * s + 2];
    g.base = static_cast<uint32_t>(total);
    g.pad = 0;
    if (g.minx > mxx || g.miny > mxy || g.minz > mxz) {
      g.dimx = g.dimy = g.dimz = 0;
    } else {
      const double dx = double(mxx) - double(g.minx) + 1.0;
      const double dy = double(mxy) - double(g.miny) + 1.0;
      const double dz = double(mxz) - double(g.minz) + 1.0;
      if (dx * dy * dz + double(total) > 2147483647.0) {
        domain = true;
        g.dimx = g.dimy = g.dimz = 0;
      } else {
        g.dimx = int(dx);
        g.dimy = int(dy);
        g.dimz = int(dz);
        total += static_cast<unsigned long long>(g.dimx) * g.dimy * g.dimz;
      }
    }
    a.grid[s] = g;
    a.bmin[3 * s + 0] = a.bmin[3 * s + 1] = a.bmin[3 * s + 2] = INT_MAX;
    a.bmax[3 * s + 0] = a.bmax[3 * s + 1] = a.bmax[3 * s + 2] = INT_MIN;
  }
  st->total_cells = total;
  st->npass = total <= 1ull ? 0 : (32 - __clz(static_cast<int>(total - 1ull)) + radix_bits - 1) / radix_bits;
  if (domain) {
    set_error(st, FLUID_ERR_DOMAIN);
  } else if (static_cast<long long>(total) > a.grid_capacity) {
    st->need_grid = total;
    set_error(st, FLUID_ERR_CAPACITY);
  }
}

__global__ void __launch_bounds__(kBlock) k_keys(StepArgs a) {
  if (failed(a.status)) return;
  const int s = blockIdx.x * kBlock + threadIdx.x;
  if (s >= a.n) return;
  const float4 x = a.x_old[s];
  float4 v = a.v_old[s];
  const int scene = __float_as_int(v.w);
  const SceneConst& c = a.sc[scene];
  const float4 p = predict(c, x, v);
  int cx, cy, cz;
  if (!cell_of(c, p, cx, cy, cz)) {
    const bool finite = isfinite(p.x) && isfinite(p.y) && isfinite(p.z);
    set_error(a.status, finite ? FLUID_ERR_DOMAIN : FLUID_ERR_NONFINITE);
    return;
  }
  a.keys[0][__float_as_int(x.w)] = cell_key(a.grid[scene], cx, cy, cz);
}

// ---------------------------------------------------------------------------
// Stable LSD radix sort, kBits-bit digits (8, 9 or 11, chosen by the autotuner),
// one kernel per pass. Pass p reads keys[p&1] (pass 0: values are the caller
// indices themselves) and writes keys[(p+1)&1]. The digit counts of every
// pass come from one read of the keys (k_radix_digits); each
// pass then ranks a tile of keys in shared memory and finds where its digits
// go by a decoupled look-back over the tiles before it: the single-pass
// prefix scan of Merrill and Garland (2016) applied per digit, as in the
// "onesweep" radix sort of Adinets and Merrill (2022).

// Look-back words, one per (tile, digit): tag (step epoch and pass) in the
// high half, then a 2-bit flag and a 30-bit count. A word whose tag is not
// the current one is not ready.
//
// The tag keeps the low 30 bits of the epoch, so tags repeat every 2^30 steps
// of one status word. Every step that runs a pass rewrites the words of all
// of that pass's tiles and digits, so a word left from an earlier step can
// carry the current tag only if it was last written exactly a multiple of
// 2^30 steps ago and no step since ran that pass over that tile (a grid that
// needed fewer passes, or a smaller particle count, for all of 2^30 steps).
// That bound -- about 12 days of back-to-back 1 ms steps -- is an accepted
// limit of a solver handle; a new handle or configure starts its own words.
constexpr uint32_t kLookAggregate = 1u;  // count = this tile's keys of the digit
constexpr uint32_t kLookPrefix = 2u;     // count = keys of the digit in tiles 0..this
constexpr int kLookSpinLimit = 1 << 22;  // then the step fails (FLUID_ERR_CUDA)
constexpr int kLookWindow = 4;           // earlier tiles read per look-back step

__device__ __forceinline__ unsigned long long look_word(uint32_t tag, uint32_t flag, uint32_t count) {
  return (static_cast<unsigned long long>(tag) << 32) | (static_cast<unsigned long long>(flag) << 30) | count;
}

__device__ __forceinline__ uint32_t look_tag(const DevStatus* st, int pass) {
  return (static_cast<uint32_t>(st->epoch) << 2) | static_cast<uint32_t>(pass);
}

// Digit counts of every pass (digit_total[pass * kBins + d]) from one read
// of the keys; grid-stride over the radix tiles. At 8-bit digits each warp
// counts into its own copy (fewer collisions on one counter).
template <int kBits>
__global__ void __launch_bounds__(kBlock) k_radix_digits(StepArgs a) {
  if (failed(a.status)) return;
  constexpr int kBins = 1 << kBits;
  constexpr int kPasses = (32 + kBits - 1) / kBits < kRadixMaxPasses ? (32 + kBits - 1) / kBits : kRadixMaxPasses;
  constexpr int kCopies = kBits <= 8 ? kBlock / 32 : 1;
  const int npass = a.status->npass;
  if (npass == 0) return;
  __shared__ uint32_t cnt[kCopies][kPasses][kBins];
  for (int i = threadIdx.x; i < kCopies * kPasses * kBins; i += kBlock) (&cnt[0][0][0])[i] = 0;
  __syncthreads();
  const int copy = kCopies > 1 ? (threadIdx.x >> 5) : 0;
  const uint32_t* keys = a.keys[0];
  for (long long base = static_cast<long long>(blockIdx.x) * kRadixTile; base < a.n;
       base += static_cast<long long>(gridDim.x) * kRadixTile) {
#pragma unroll
    for (int r = 0; r < kRadixItems; ++r) {
      const long long idx = base + r * kBlock + threadIdx.x;
      if (idx >= a.n) continue;
      const uint32_t key = keys[idx];
      for (int p = 0; p < npass && p < kPasses; ++p)
        atomicAdd(&cnt[copy][p][(key >> (kBits * p)) & (kBins - 1u)], 1u);
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < npass * kBins && i < kPasses * kBins; i += kBlock) {
    uint32_t v = 0;
#pragma unroll
    for (int c = 0; c < kCopies; ++c) v += (&cnt[c][0][0])[i];
    if (v) atomicAdd(&a.digit_total[i], v);
  }
}

// Exclusive prefix over the kBins digit counts `tot` into starts[] (shared),
// by the whole block; ends with a barrier.
template <int kBits, int kThreads = kBlock>
__device__ __forceinline__ void digit_starts(const uint32_t* __restrict__ tot, uint32_t* starts) {
  constexpr int kBins = 1 << kBits;
  constexpr int kPer = (kBins + kThreads - 1) / kThreads;  // contiguous digits per thread
  __shared__ uint32_t warp_sums[kThreads / 32];
  uint32_t v[kPer];
  uint32_t sum = 0;
#pragma unroll
  for (int k = 0; k < kPer; ++k) {
    const int d = threadIdx.x * kPer + k;
    v[k] = d < kBins ? tot[d] : 0u;
    sum += v[k];
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t inc = sum;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(kFull, inc, o);
    if (lane >= o) inc += y;
  }
  if (lane == 31) warp_sums[warp] = inc;
  __syncthreads();
  uint32_t before = inc - sum;
  for (int w = 0; w < warp; ++w) before += warp_sums[w];
#pragma unroll
  for (int k = 0; k < kPer; ++k) {
    const int d = threadIdx.x * kPer + k;
    if (d < kBins) starts[d] = before;
    before += v[k];
  }
  __syncthreads();
}

// One pass: tiles are taken in launch order from a counter (so every tile a
// tile waits for has started, and the waits always end), ranked in shared
// memory, placed by the look-back, and scattered.
template <int kBits, int kSortThreads = sort_threads(kBits)>
__global__ void __launch_bounds__(kSortThreads) k_radix_onesweep(StepArgs a, int pass) {
  constexpr int kBins = 1 << kBits;
  constexpr int kItems = kRadixTile / kSortThreads;  // keys per thread
  // Per-warp digit counts; at most kRadixTile = 4096 per tile, so 16 bits
  // hold them where 32-bit counters would not fit in shared memory.
  using Count = typename std::conditional<(kBits <= 8), uint32_t, uint16_t>::type;
  __shared__ Count wcnt[kSortThreads / 32][kBins];
  __shared__ uint32_t goff[kBins];  // digit starts, then this tile's first slot per digit
  __shared__ int s_tile, s_skip;
  if (threadIdx.x == 0) {
    s_skip = (failed(a.status) || pass >= a.status->npass) ? 1 : 0;
    s_tile = s_skip ? 0 : atomicAdd(&a.radix_next[pass], 1);
  }
  __syncthreads();
  if (s_skip) return;
  const int tile = s_tile;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int i = threadIdx.x; i < (kSortThreads / 32) * kBins; i += kSortThreads) (&wcnt[0][0])[i] = 0;
  digit_starts<kBits, kSortThreads>(a.digit_total + pass * kBins, goff);
  const uint32_t* kin = a.keys[pass & 1];
  const int* vin = a.vals[pass & 1];
  uint32_t* kout = a.keys[(pass + 1) & 1];
  int* vout = a.vals[(pass + 1) & 1];
  const int shift = kBits * pass;
  // Warp w ranks its contiguous 32*kItems keys in order, 32 at a time.
  const long long base = static_cast<long long>(tile) * kRadixTile + warp * (32 * kItems);
  uint32_t key[kItems];
  int val[kItems];
  int dig[kItems];
  uint32_t rank[kItems];
#pragma unroll
  for (int r = 0; r < kItems; ++r) {
    const long long idx = base + r * 32 + lane;
    const bool ok = idx < a.n;
    key[r] = ok ? kin[idx] : 0u;
    val[r] = ok ? (pass == 0 ? static_cast<int>(idx) : vin[idx]) : 0;
    const int d = ok ? static_cast<int>((key[r] >> shift) & (kBins - 1u)) : kBins;
    dig[r] = d;
    const unsigned peers = __match_any_sync(kFull, d);
    const uint32_t before = __popc(peers & lanemask_lt(lane));
    const uint32_t run = (d < kBins) ? static_cast<uint32_t>(wcnt[warp][d]) : 0u;
    __syncwarp();
    if (d < kBins && before == 0) wcnt[warp][d] = static_cast<Count>(run + __popc(peers));
    __syncwarp();
    rank[r] = run + before;
  }
  __syncthreads();
  // Every digit's count goes out first (tile 0's as a prefix), so a tile
  // behind this one never waits on this tile's own look-back. Thread t owns
  // digits t, t + kSortThreads, ... in both loops.
  constexpr int kOwn = (kBins + kSortThreads - 1) / kSortThreads;
  const uint32_t tag = look_tag(a.status, pass);
  unsigned long long* look = a.look + static_cast<long long>(tile) * kBins;
  uint32_t runs[kOwn];
#pragma unroll
  for (int k = 0; k < kOwn; ++k) {
    const int d = threadIdx.x + k * kSortThreads;
    runs[k] = 0;
    if (d >= kBins) continue;
    uint32_t run = 0;
#pragma unroll
    for (int w = 0; w < kSortThreads / 32; ++w) {
      const uint32_t t = wcnt[w][d];
      wcnt[w][d] = static_cast<Count>(run);
      run += t;
    }
    runs[k] = run;
    *(volatile unsigned long long*)(look + d) = look_word(tag, tile == 0 ? kLookPrefix : kLookAggregate, run);
  }
  bool timed_out = false;
#pragma unroll
  for (int k = 0; k < kOwn; ++k) {
    const int d = threadIdx.x + k * kSortThreads;
    if (d >= kBins) continue;
    uint32_t excl = 0;
    if (tile > 0) {
      // kLookWindow earlier tiles' words read at once, used nearest first
      // up to the first one not ready yet (polled again) or a prefix.
      int j = tile - 1;
      int spins = 0;
      for (;;) {
        unsigned long long w[kLookWindow];
#pragma unroll
        for (int u = 0; u < kLookWindow; ++u)
          w[u] = (j - u >= 0) ? *(volatile const unsigned long long*)(a.look + static_cast<long long>(j - u) * kBins + d)
                              : 0ull;
        int used = 0;
        bool done = false;
#pragma unroll
        for (int u = 0; u < kLookWindow; ++u) {
          if (used != u || done) break;
          const uint32_t flag = static_cast<uint32_t>(w[u] >> 30) & 3u;
          if (static_cast<uint32_t>(w[u] >> 32) != tag || flag == 0u) break;
          excl += static_cast<uint32_t>(w[u]) & 0x3fffffffu;
          used = u + 1;
          done = flag == kLookPrefix;  // tile 0 always ends the walk with a prefix
        }
        if (done) break;
        if (used == 0) {
          if (++spins > kLookSpinLimit) {
            timed_out = true;
            break;
          }
          if (spins > 64) __nanosleep(64);
        }
        j -= used;
      }
      *(volatile unsigned long long*)(look + d) = look_word(tag, kLookPrefix, excl + runs[k]);
    }
    goff[d] += excl;
  }
  if (timed_out) set_error(a.status, FLUID_ERR_CUDA);
  __syncthreads();
#pragma unroll
  for (int r = 0; r < kItems; ++r) {
    const int d = dig[r];
    if (d < kBins) {
      const uint32_t pos = goff[d] + wcnt[warp][d] + rank[r];
      if (pos < static_cast<uint32_t>(a.n)) {
        kout[pos] = key[r];
        vout[pos] = val[r];
      } else {
        set_error(a.status, FLUID_ERR_CUDA);
      }
    }
  }
}

// The whole sort in one block, for a batch of at most one tile (kRadixTile
// keys): every 8-bit pass ranks the keys as k_radix_onesweep does (warp-
// private digit counts in key order, then the warps' offsets per digit) and
// places them through shared memory, the keys staying in registers between
// passes; no digit-count kernel, no look-back, one launch instead of one per
// pass. The result is the same stable order, written where k_reorder reads
// the last pass's output (keys/vals[npass & 1] for the plan's pass count).
__global__ void __launch_bounds__(kBlock) k_radix_tile(StepArgs a) {
  constexpr int kBits = 8, kBins = 1 << kBits;
  static_assert(kBins == kBlock, "thread t owns digit t");
  __shared__ uint32_t wcnt[kBlock / 32][kBins];
  __shared__ uint32_t total[kBins], start[kBins];
  __shared__ uint32_t sk[kRadixTile];
  __shared__ int sv[kRadixTile];
  __shared__ int s_skip;
  if (threadIdx.x == 0) s_skip = (failed(a.status) || a.status->npass == 0) ? 1 : 0;
  __syncthreads();
  if (s_skip) return;
  const DevStatus* st = a.status;
  const unsigned long long cells = st->total_cells;
  const int bits = 32 - __clz(static_cast<int>(cells - 1ull));
  const int passes = (bits + kBits - 1) / kBits;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int base = warp * (32 * kRadixItems);  // warp w holds keys [base, base + 32 kRadixItems)
  uint32_t key[kRadixItems];
  int val[kRadixItems];
#pragma unroll
  for (int r = 0; r < kRadixItems; ++r) {
    const int idx = base + r * 32 + lane;
    const bool ok = idx < a.n;
    key[r] = ok ? a.keys[0][idx] : 0xffffffffu;  // padding sorts last and is not written
    val[r] = ok ? idx : -1;
  }
  for (int pass = 0; pass < passes; ++pass) {
    const int shift = kBits * pass;
    for (int i = threadIdx.x; i < (kBlock / 32) * kBins; i += kBlock) (&wcnt[0][0])[i] = 0;
    __syncthreads();
    uint32_t rank[kRadixItems];
    int dig[kRadixItems];
#pragma unroll
    for (int r = 0; r < kRadixItems; ++r) {
      const int d = static_cast<int>((key[r] >> shift) & (kBins - 1u));
      dig[r] = d;
      const unsigned peers = __match_any_sync(kFull, d);
      const uint32_t before = __popc(peers & lanemask_lt(lane));
      const uint32_t run = wcnt[warp][d];
      __syncwarp();
      if (before == 0) wcnt[warp][d] = run + __popc(peers);
      __syncwarp();
      rank[r] = run + before;
    }
    __syncthreads();
    // Thread t owns digit t: the warps' offsets within it, and its total.
    {
      const int d = threadIdx.x;  // kBlock == kBins
      uint32_t run = 0;
#pragma unroll
      for (int w = 0; w < kBlock / 32; ++w) {
        const uint32_t t = wcnt[w][d];
        wcnt[w][d] = run;
        run += t;
      }
      total[d] = run;
    }
    __syncthreads();
    digit_starts<kBits>(total, start);
#pragma unroll
    for (int r = 0; r < kRadixItems; ++r) {
      const uint32_t pos = start[dig[r]] + wcnt[warp][dig[r]] + rank[r];
      sk[pos] = key[r];
      sv[pos] = val[r];
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kRadixItems; ++r) {
      key[r] = sk[base + r * 32 + lane];
      val[r] = sv[base + r * 32 + lane];
    }
    __syncthreads();
  }
  uint32_t* kout = a.keys[st->npass & 1];
  int* vout = a.vals[st->npass & 1];
#pragma unroll
  for (int r = 0; r < kRadixItems; ++r) {
    const int idx = base + r * 32 + lane;
    if (idx < a.n) {
      kout[idx] = key[r];
      vout[idx] = val[r];
    }
  }
}

// ---------------------------------------------------------------------------
// Reorder into cell order and cell table.

__global__ void __launch_bounds__(kBlock) k_reorder(StepArgs a) {
  if (failed(a.status)) return;
  const int s = blockIdx.x * kBlock + threadIdx.x;
  const int lane = threadIdx.x & 31;
  const int npass = a.status->npass;
  const uint32_t* ks = sorted_keys(a, npass);
  const bool ok = s < a.n;
  const uint32_t key = ok ? ks[s] : 0xffffffffu;
  // Neighbouring keys through the warp; warp-edge lanes read memory.
  uint32_t prev = __shfl_up_sync(kFull, key, 1);
  uint32_t next = __shfl_down_sync(kFull, key, 1);
  if (!ok) return;
  if (lane == 0) prev = (s > 0) ? ks[s - 1] : ~key;
  if (lane == 31 || s + 1 >= a.n) next = (s + 1 < a.n) ? ks[s + 1] : ~key;
  int* table = reinterpret_cast<int*>(a.table);
  if (prev != key) table[2ll * key] = s;
  if (next != key) table[2ll * key + 1] = s + 1;

  const int orig = npass ? a.vals[npass & 1][s] : s;
  const int old = a.slot_old[orig];
  const float4 x = a.x_old[old];
  float4 v = a.v_old[old];
  const int scene = __float_as_int(v.w);
  const SceneConst& c = a.sc[scene];
  const float4 p = predict(c, x, v);
  a.x[s] = x;
  a.v[s] = v;
  a.p[0][s] = p;
  a.slot[orig] = s;
  if (c.iterations == 0) a.rho[s] = a.rho_old[old];
}

// ---------------------------------------------------------------------------
// Neighbour lists.

// Calls f(j, pos[j], ok) for j in [lo, hi), ok false for j == self (kSkip); kFetch
// records loaded before any is used. Lanes of a warp whose particles share a
// cell walk the same j together, so each load is a broadcast.
template <int kFetch, bool kSkip, typename F>
__device__ __forceinline__ void scan_range(const float4* __restrict__ pos, int lo, int hi, int self, F& f) {
  int j = lo;
  for (; j + kFetch <= hi; j += kFetch) {
    float4 q[kFetch];
#pragma unroll
    for (int u = 0; u < kFetch; ++u) q[u] = __ldg(pos + j + u);
#pragma unroll
    for (int u = 0; u < kFetch; ++u) f(j + u, q[u], !kSkip || j + u != self);
  }
  for (; j < hi; ++j) f(j, __ldg(pos + j), !kSkip || j != self);
}

// Visits the 27 cells around p in the reference's order (core.cpp:211-243),
// calling f(j, q_j, ok) for each particle of them; ok is false for j == i
// (tested in the centre cell only). Cell keys advance incrementally along x;
// candidates are fetched kFetch at a time (issued before any is tested,
// tested in order).
template <int kFetch, typename F>
__device__ __forceinline__ void for_each_candidate(const StepArgs& a, const uint32_t* ks, const GridInfo& g,
                                                   const SceneConst& c, int i, const float4 p,
                                                   const float4* __restrict__ pos, F&& f) {
  int cx, cy, cz;
  cell_of(c, p, cx, cy, cz);
  const int xstride = g.dimy * g.dimz;
  for (int oz = -1; oz <= 1; ++oz) {
    const int z = cz + oz;
    if (z < g.minz || z >= g.minz + g.dimz) continue;
    for (int oy = -1; oy <= 1; ++oy) {
      const int y = cy + oy;
      if (y < g.miny || y >= g.miny + g.dimy) continue;
      // The row's three cell ranges: table entries, then their validating
      // keys, each three loads in flight, then the scans in x order. The
      // table is not cleared between steps; an entry left from an earlier
      // step is rejected because the first slot of a live entry holds that
      // cell's key this step.
      const uint32_t key0 = cell_key(g, cx - 1, y, z);
      int2 e[3];
      uint32_t kk[3];
#pragma unroll
      for (int t = 0; t < 3; ++t) {
        const int xx = cx - 1 + t;
        const bool in = xx >= g.minx && xx < g.minx + g.dimx;
        e[t] = in ? a.table[key0 + static_cast<uint32_t>(t * xstride)] : make_int2(0, 0);
      }
#pragma unroll
      for (int t = 0; t < 3; ++t) {
        if (e[t].x < 0 || e[t].x >= e[t].y || e[t].y > a.n) e[t] = make_int2(0, 0);
        kk[t] = e[t].x < e[t].y ? __ldg(ks + e[t].x) : 0u;
      }
#pragma unroll
      for (int t = 0; t < 3; ++t) {
        if (e[t].x >= e[t].y || kk[t] != key0 + static_cast<uint32_t>(t * xstride)) continue;
        if (oz == 0 && oy == 0 && t == 1) scan_range<kFetch, true>(pos, e[t].x, e[t].y, i, f);
        else scan_range<kFetch, false>(pos, e[t].x, e[t].y, i, f);
      }
    }
  }
}

// Lambda from the accumulated sums (core.cpp:319-328).
__device__ __forceinline__ float finish_lambda(const SceneConst& c, float rho, float gsx, float gsy, float gsz,
                                               float sum_g2, float& rho_out) {
  rho = rho + c.w0;
  rho = rho * c.mass;
  rho_out = rho;
  const float C = rho * c.inv_density - 1.0f;
  const float ix = c.grad_scale * gsx;
  const float iy = c.grad_scale * gsy;
  const float iz = c.grad_scale * gsz;
  sum_g2 += ix * ix + iy * iy + iz * iz;
  return -C / (sum_g2 + c.epsilon);
}

// Per-neighbour density / gradient terms (core.cpp:300-316).
struct LambdaAcc {
  float rho = 0.0f, gsx = 0.0f, gsy = 0.0f, gsz = 0.0f, sum_g2 = 0.0f;
  template <bool kIeee = false>
  __device__ __forceinline__ void add(const SceneConst& c, float dx, float dy, float dz, float r2) {
    rho += poly6(c, r2);
    const float gf = spiky(c, clamped_r<kIeee>(c, r2));
    const float gx = gf * dx, gy = gf * dy, gz = gf * dz;
    gsx += gx;
    gsy += gy;
    gsz += gz;
    const float ng = -c.grad_scale;
    const float jx = ng * gx, jy = ng * gy, jz = ng * gz;
    sum_g2 += jx * jx + jy * jy + jz * jz;
  }
  // Entries a and b (in list order) relative to p, each added only when
  // r2 < h2: the same operations as the membership test plus add() on a,
  // then on b, with the per-entry terms formed in paired arithmetic.
  // Returns which of a (bit 0) and b (bit 1) were within h.
  template <bool kIeee = false>
  __device__ __forceinline__ unsigned add_pair(const SceneConst& c, const float2 px, const float2 py,
                                               const float2 pz, const float4 qa, const float4 qb) {
    const float2 nz = f2(c.neg_zero);
    const PairGeom g = pair_geom(px, py, pz, qa, qb, nz);
    const bool oka = g.r2.x < c.h2, okb = g.r2.y < c.h2;
    if (!oka && !okb) return 0u;
    const float2 w = poly6_pair(c, g.r2, nz);
    const float2 gf = spiky_pair<kIeee>(c, g.r2, nz);
    const float2 gx = pmul(gf, g.dx, nz), gy = pmul(gf, g.dy, nz), gz = pmul(gf, g.dz, nz);
    const float2 ng = f2(-c.grad_scale);
    const float2 jx = pmul(ng, gx, nz), jy = pmul(ng, gy, nz), jz = pmul(ng, gz, nz);
    const float2 t = padd(padd(pmul(jx, jx, nz), pmul(jy, jy, nz)), pmul(jz, jz, nz));
    if (oka) {
      rho += w.x;
      gsx += gx.x;
      gsy += gy.x;
      gsz += gz.x;
      sum_g2 += t.x;
    }
    if (okb) {
      rho += w.y;
      gsx += gx.y;
      gsy += gy.y;
      gsz += gz.y;
      sum_g2 += t.y;
    }
    return (oka ? 1u : 0u) | (okb ? 2u : 0u);
  }
};

// All-pairs candidates (core.cpp:248-268, use_uniform_grid == 0): every other
// particle of the scene in ascending caller index, as the reference's
// fallback visits them. O(N^2) per scene; meant for small scenes.
template <typename F>
__device__ __forceinline__ void for_each_pair_candidate(const StepArgs& a, const SceneConst& c, int i,
                                                        const float4* __restrict__ pos, F&& f) {
  for (int o = c.first_slot; o < c.first_slot + c.count; ++o) {
    const int j = a.slot[o];
    if (j == i) continue;
    f(j, pos[j]);
  }
}

// Neighbour lists in one scan (core.cpp:205-247). Each lane stages its first
// stage_rows list entries in shared memory while it scans. The staging takes no
// branch on the r2 test: every candidate is stored in the lane's next free
// row, and the count advances only when the candidate is within h, so a
// rejected candidate is overwritten by the next one (row stage_rows is a spare
// that absorbs the stores past the staged rows). At ~13 % acceptance this
// took the lattice build from 0.285 to 0.260 ms per 1M step and the
// collapsed 125k build from 0.96 to 0.80 ms against a branch around the
// store. The block then claims its warps' 32-wide
// slices with one atomic on the list cursor (placement varies run to run,
// every list's content and order do not) and writes the staged entries out
// as coalesced 128-byte rows. A warp with a longer list (kSliceOverflow in
// slice_fmt[w]) then scans its candidates a second time and writes the
// entries past the staged rows straight into its slice: the same work a
// separate pass over all particles did after the build, without that pass's
// launch (14 us per 1M lattice step with nothing to do; 2 ms less per 1M
// collapsed step).
// kRows: the staged rows when fixed at compile time (the default, which the
// lattice phase uses), 0 to read them from the plan (a.stage_rows).
template <int kRows>
__global__ void __launch_bounds__(kMaxBuildBlock) k_nbr_build(StepArgs a) {
  extern __shared__ int stage[];
  // Other blocks of this launch may set the status (capacity) while this
  // one starts: read it once for the whole block, so either every warp
  // returns here or every warp reaches the barriers and the slice claim
  // below (a warp left behind by an early return of thread 0's warp would
  // read an unset block_base).
  __shared__ int block_failed;
  if (threadIdx.x == 0) block_failed = failed(a.status) ? 1 : 0;
  __syncthreads();
  if (block_failed) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int rows = kRows > 0 ? kRows : a.stage_rows;
  int* mine = stage + warp * ((rows + 1) * 32) + lane;  // entry k at mine[32 k]
  int count = 0;
  const bool live = i < a.n;
  const uint32_t* ks = sorted_keys(a, a.status->npass);
  const float4 p = live ? a.p[0][i] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  const int scene = __float_as_int(p.w);
  const SceneConst& c = a.sc[scene];
  const GridInfo g = a.grid[scene];
  const float h2 = c.h2;
  if (live) {
    auto test = [&](int j, const float4 q, bool ok) {
      const bool in = dist2(p.x - q.x, p.y - q.y, p.z - q.z) < h2 && ok;
      mine[32 * min(count, rows)] = j;
      count += in ? 1 : 0;
    };
    if (c.all_pairs) for_each_pair_candidate(a, c, i, a.p[0], [&](int j, const float4 q) { test(j, q, true); });
    else for_each_candidate<4>(a, ks, g, c, i, p, a.p[0], test);
    a.cnt[i] = count;
  }
  const int mx = __reduce_max_sync(kFull, count);
  const unsigned sum = __reduce_add_sync(kFull, static_cast<unsigned>(count));
  // A warp whose lists are all staged and whose entries all lie within
  // 32768 slots of its anchor writes 16-bit offsets (half the bytes for
  // every list pass to read; the whole 1M lattice qualifies). Its slice is
  // rounded up to whole 128-byte lines.
  const int anchor = (i - lane) - kSliceAnchorBack;
  bool near = true;
  if (a.list16 && mx <= rows) {
    for (int k = 0; k < count; ++k) near = near && static_cast<unsigned>(mine[32 * k] - anchor) <= 0xffffu;
  }
  const bool slim = __all_sync(kFull, near) && a.list16 && mx <= rows;
  const int ints = slim ? 32 * ((mx + 1) / 2) : 32 * mx;  // the warp's slice
  __shared__ int wints[kMaxBuildBlock / 32];
  __shared__ unsigned long long block_base;
  __shared__ int block_ok;
  const bool warp_live = (i - lane) < a.n;
  if (lane == 0) {
    wints[warp] = warp_live ? ints : 0;
    if (warp_live) {
      if (sum) atomicAdd(&a.status->pairs, static_cast<unsigned long long>(sum));
      if (mx) atomicMax(&a.status->nbr_max, mx);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long total = 0;
    for (int w = 0; w < static_cast<int>(blockDim.x / 32); ++w) total += static_cast<unsigned long long>(wints[w]);
    const unsigned long long base = atomicAdd(&a.status->cursor, total);
    block_ok = base + total <= static_cast<unsigned long long>(a.nbr_capacity);
    if (!block_ok) set_error(a.status, FLUID_ERR_CAPACITY);
    block_base = base;
  }
  __syncthreads();
  if (!warp_live || !block_ok) return;
  unsigned long long off = block_base;
  for (int w = 0; w < warp; ++w) off += static_cast<unsigned long long>(wints[w]);
  if (slim) {
    unsigned short* out = reinterpret_cast<unsigned short*>(a.nbr + off) + lane;
    for (int k = 0; k < mx; ++k)
      if (k < count) out[32 * k] = static_cast<unsigned short>(mine[32 * k] - anchor);
  } else {
    int* out = a.nbr + off + lane;
    const int staged = mx < rows ? mx : rows;
    for (int k = 0; k < staged; ++k)
      if (k < count) out[32ll * k] = mine[32 * k];
  }
  if (lane == 0) {
    a.wbase[i >> 5] = static_cast<long long>(off);
    a.depth[i >> 5] = mx;
    a.slice_fmt[i >> 5] = (mx > rows ? kSliceOverflow : 0) | (slim ? kSlice16 : 0);
  }
  if (mx > rows && live) {
    // Entries rows and above: a second scan, written straight into the slice.
    int* out = a.nbr + off + lane;
    int k = 0;
    auto rest = [&](int j, const float4 q, bool ok) {
      if (ok && dist2(p.x - q.x, p.y - q.y, p.z - q.z) < h2) {
        if (k >= rows && k < mx) out[32ll * k] = j;
        ++k;
      }
    };
    if (c.all_pairs) for_each_pair_candidate(a, c, i, a.p[0], [&](int j, const float4 q) { rest(j, q, true); });
    else for_each_candidate<4>(a, ks, g, c, i, p, a.p[0], rest);
  }
}

// ---------------------------------------------------------------------------
// Jacobi passes over the lists.

// Rows ahead of its current position at which a walk over a long list asks
// the L2 for the list (one prefetch per row, on the lane's own entry; the
// warp's 32 entries of a row share one 128-byte line). The walk's own index
// loads run one group of entries ahead, which is enough for the lattice's
// ~28-entry lists but leaves a collapsed state's thousands of rows per warp
// streaming from DRAM one group at a time.
constexpr int kListAhead = 32;

__device__ __forceinline__ void prefetch_row(const void* p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }

// A lane's list in its warp's slice, in either row format: entry(k) is list
// entry k (streamed with the evict-first hint: each pass reads a row once),
// row(k) its address, from(k0) the list from entry k0 on.
struct List32 {
  const int* __restrict__ p;  // the lane's entry in row 0
  __device__ __forceinline__ int entry(long long k) const { return __ldcs(p + 32 * k); }
  __device__ __forceinline__ const void* row(long long k) const { return p + 32 * k; }
  __device__ __forceinline__ List32 from(int k0) const { return {p + 32ll * k0}; }
};
struct List16 {
  const unsigned short* __restrict__ p;
  int anchor;  // 32 w - kSliceAnchorBack
  __device__ __forceinline__ int entry(long long k) const { return anchor + static_cast<int>(__ldcs(p + 32 * k)); }
  __device__ __forceinline__ const void* row(long long k) const { return p + 32 * k; }
  __device__ __forceinline__ List16 from(int k0) const { return {p + 32ll * k0, anchor}; }
};

// Calls f(list) with lane i's list in the format of its warp's slice (the
// same for every lane of a warp, so the branch does not split warps).
template <typename F>
__device__ __forceinline__ void with_list(const StepArgs& a, int i, F&& f) {
  const int w = i >> 5;
  const long long base = a.wbase[w];
  if (a.slice_fmt[w] & kSlice16) {
    f(List16{reinterpret_cast<const unsigned short*>(a.nbr + base) + (i & 31), (i & ~31) - kSliceAnchorBack});
  } else {
    f(List32{a.nbr + base + (i & 31)});
  }
}

// with_list for the kernels with several lanes per particle, called by every
// lane of the warp (their walk shuffles over the whole warp, so the branch
// must not split it): the format is that of the warp's first particle, and
// the warp's particles, consecutive and at most 32, all lie in that
// particle's slice. A lane past the last particle gets an empty list.
template <typename F>
__device__ __forceinline__ void with_list_lanes(const StepArgs& a, int i, bool valid, F&& f) {
  const int i0 = __shfl_sync(kFull, i, 0);
  const int fmt = i0 < a.n ? a.slice_fmt[i0 >> 5] : 0;
  const long long base = valid ? a.wbase[i >> 5] : 0;
  if (fmt & kSlice16) {
    f(List16{reinterpret_cast<const unsigned short*>(a.nbr + base) + (valid ? (i & 31) : 0),
             (i & ~31) - kSliceAnchorBack});
  } else {
    f(List32{a.nbr + base + (valid ? (i & 31) : 0)});
  }
}

// Walks this lane's list entries k = 0..n-1 in order. kUnroll records are
// fetched before any is used, and the next kUnroll list indices are fetched
// while the current records are processed, so every warp keeps several
// independent gathers in flight and the index latency stays hidden; the body
// still sees the entries in list order, so sums accumulate in the
// reference's order.
template <int kUnroll, typename L, typename Load, typename Body>
__device__ __forceinline__ void for_each_neighbor(const L& list, int n, Load&& load, Body&& body) {
  using Rec = decltype(load(0));
  int k = 0;
  int j[kUnroll];
  if (kUnroll <= n) {
#pragma unroll
    for (int u = 0; u < kUnroll; ++u) j[u] = list.entry(u);
  }
  for (; k + kUnroll <= n; k += kUnroll) {
    Rec r[kUnroll];
#pragma unroll
    for (int u = 0; u < kUnroll; ++u) r[u] = load(j[u]);
    if (k + 2 * kUnroll <= n) {
#pragma unroll
      for (int u = 0; u < kUnroll; ++u) j[u] = list.entry(k + kUnroll + u);
    }
    if (k + kListAhead + kUnroll <= n) {
#pragma unroll
      for (int u = 0; u < kUnroll; ++u) prefetch_row(list.row(k + kListAhead + u));
    }
#pragma unroll
    for (int u = 0; u < kUnroll; ++u) body(r[u]);
  }
  for (; k < n; ++k) body(load(list.entry(k)));
}

// for_each_neighbor for bodies that take two consecutive entries at once
// (a then b, in list order); an odd last entry goes to body1. kUnroll >= 2.
template <int kUnroll, typename L, typename Load, typename Body2, typename Body1>
__device__ __forceinline__ void for_each_neighbor_pair(const L& list, int n, Load&& load, Body2&& body2,
                                                       Body1&& body1) {
  static_assert(kUnroll % 2 == 0, "entries are consumed in pairs");
  using Rec = decltype(load(0));
  int k = 0;
  int j[kUnroll];
  if (kUnroll <= n) {
#pragma unroll
    for (int u = 0; u < kUnroll; ++u) j[u] = list.entry(u);
  }
  for (; k + kUnroll <= n; k += kUnroll) {
    Rec r[kUnroll];
#pragma unroll
    for (int u = 0; u < kUnroll; ++u) r[u] = load(j[u]);
    if (k + 2 * kUnroll <= n) {
#pragma unroll
      for (int u = 0; u < kUnroll; ++u) j[u] = list.entry(k + kUnroll + u);
    }
    if (k + kListAhead + kUnroll <= n) {
#pragma unroll
      for (int u = 0; u < kUnroll; ++u) prefetch_row(list.row(k + kListAhead + u));
    }
#pragma unroll
    for (int u = 0; u < kUnroll; u += 2) body2(r[u], r[u + 1]);
  }
  for (; k + 2 <= n; k += 2) {
    const Rec ra = load(list.entry(k)), rb = load(list.entry(k + 1));
    body2(ra, rb);
  }
  if (k < n) body1(load(list.entry(k)));
}

struct PosVel {
  float4 x, v;
};

// Live bits of a list's first kLiveEntries entries at one set of positions
// (the committed ones): bit k is 1 unless entry k is out of range (r2 >= h2)
// there. XSPH, which tests every entry at those positions, records them
// (for_each_neighbor_pair_rec); the vorticity passes at the same positions
// gather and evaluate only the live ones among those entries
// (for_each_live_then), the rest as usual.
constexpr int kLiveEntries = 64;

__device__ __forceinline__ void store_live(uint32_t* live, int n, int i, unsigned long long bits) {
  live[i] = static_cast<uint32_t>(bits);
  live[n + i] = static_cast<uint32_t>(bits >> 32);
}

// for_each_neighbor_pair whose bodies return which entries were within h
// (body2: bit 0 for a, bit 1 for b; body1: a bool); returns the live bits of
// the first kLiveEntries entries. Entries past those go through the plain
// walker.
template <int kUnroll, typename L, typename Load, typename Body2, typename Body1>
__device__ __forceinline__ unsigned long long for_each_neighbor_pair_rec(const L& list, int n, Load&& load,
                                                                         Body2&& body2, Body1&& body1) {
  static_assert(kUnroll % 2 == 0 && kLiveEntries % kUnroll == 0, "entries are consumed in pairs");
  using Rec = decltype(load(0));
  const int head = n < kLiveEntries ? n : kLiveEntries;
  unsigned long long bits = 0ull;
  int k = 0;
  int j[kUnroll];
  if (kUnroll <= head) {
#pragma unroll
    for (int u = 0; u < kUnroll; ++u) j[u] = list.entry(u);
  }
  for (; k + kUnroll <= head; k += kUnroll) {
    Rec r[kUnroll];
#pragma unroll
    for (int u = 0; u < kUnroll; ++u) r[u] = load(j[u]);
    if (k + 2 * kUnroll <= head) {
#pragma unroll
      for (int u = 0; u < kUnroll; ++u) j[u] = list.entry(k + kUnroll + u);
    }
    unsigned long long got = 0ull;
#pragma unroll
    for (int u = 0; u < kUnroll; u += 2) got |= static_cast<unsigned long long>(body2(r[u], r[u + 1])) << u;
    bits |= got << k;
  }
  for (; k + 2 <= head; k += 2) {
    const Rec ra = load(list.entry(k)), rb = load(list.entry(k + 1));
    bits |= static_cast<unsigned long long>(body2(ra, rb)) << k;
  }
  if (k < head && body1(load(list.entry(k)))) bits |= 1ull << k;
  if (n > kLiveEntries) for_each_neighbor_pair<kUnroll>(list.from(kLiveEntries), n - kLiveEntries, load, body2, body1);
  return bits;
}

// The first kLiveEntries entries one at a time, each read from the list and
// gathered only where its live bit is set (a dead entry costs no memory
// access); a dead entry reaches the body as `dead`, a record no particle is
// within h of, which the body rejects exactly as it would the real one
// (r2 < h2 fails). The remaining entries go through for_each_neighbor_pair.
// Sums accumulate in list order either way.
template <int kUnroll, typename L, typename Load, typename Rec, typename Body2, typename Body1>
__device__ __forceinline__ void for_each_live_then(const L& list, int n, unsigned long long bits, Load&& load,
                                                   const Rec dead, Body2&& body2, Body1&& body1) {
  const int head = n < kLiveEntries ? n : kLiveEntries;
  unsigned long long m = head < kLiveEntries ? bits & ((1ull << head) - 1ull) : bits;
  if (m) {
    // Live entries only, in order, the next one's record loaded while the
    // current one is used.
    int k = __ffsll(static_cast<long long>(m)) - 1;
    m &= m - 1ull;
    auto r = load(list.entry(k));
    while (m) {
      const int kn = __ffsll(static_cast<long long>(m)) - 1;
      m &= m - 1ull;
      const auto rn = load(list.entry(kn));
      body1(r);
      r = rn;
    }
    body1(r);
  }
  if (n > kLiveEntries) {
    if constexpr (kUnroll == 1) {
      for_each_neighbor<1>(list.from(kLiveEntries), n - kLiveEntries, load, body1);
    } else {
      for_each_neighbor_pair<kUnroll>(list.from(kLiveEntries), n - kLiveEntries, load, body2, body1);
    }
  }
}

// kLiveOut: record the live bits of these positions for the delta pass
// (iterations after the first; the first runs at the positions the lists
// were built from, where every entry is live).
template <int U, bool kLiveOut, bool kIeee = false>
__global__ void __launch_bounds__(kMaxBlock, FGB_LIST_MIN_BLOCKS) k_lambda(StepArgs a, int in) {
  if (failed(a.status)) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const float4* __restrict__ pos = a.p[in];
  const float4 p = pos[i];
  const SceneConst& c = a.sc[__float_as_int(p.w)];
  const int n = a.cnt[i];
  const float h2 = c.h2;
  LambdaAcc acc;
  auto one = [&](const float4 q) {
    const float dx = p.x - q.x, dy = p.y - q.y, dz = p.z - q.z;
    const float r2 = dist2(dx, dy, dz);
    if (r2 < h2) acc.add<kIeee>(c, dx, dy, dz, r2);
    return r2 < h2;
  };
  auto load = [&](int j) { return __ldg(pos + j); };
  with_list(a, i, [&](const auto& list) {
    if constexpr (U == 1) {
      if constexpr (kLiveOut) {
        unsigned long long bits = 0ull;
        int k = 0;
        for_each_neighbor<1>(list, n, load, [&](const float4 q) {
          if (one(q) && k < kLiveEntries) bits |= 1ull << k;
          ++k;
        });
        store_live(a.live, a.n, i, bits);
      } else {
        for_each_neighbor<1>(list, n, load, one);
      }
    } else {
      const float2 px = f2(p.x), py = f2(p.y), pz = f2(p.z);
      auto two = [&](const float4 qa, const float4 qb) { return acc.add_pair<kIeee>(c, px, py, pz, qa, qb); };
      if constexpr (kLiveOut) store_live(a.live, a.n, i, for_each_neighbor_pair_rec<U>(list, n, load, two, one));
      else for_each_neighbor_pair<U>(list, n, load, two, one);
    }
  });
  float rho;
  const float lam = finish_lambda(c, acc.rho, acc.gsx, acc.gsy, acc.gsz, acc.sum_g2, rho);
  a.lambda[i] = lam;
  a.rho[i] = rho;
  a.pl[i] = make_float4(p.x, p.y, p.z, lam);
}

// Commit v = (p - x)/dt, x = p (core.cpp:414-421); restitution when this is
// the step's last velocity write. Ahead of XSPH (to_v2) it also writes the
// record XSPH gathers per neighbour, {x.xyz, m / rho} into xr: the
// per-neighbour factor of core.cpp:446-447, the same value for every i.
__device__ __forceinline__ void commit(const StepArgs& a, const SceneConst& c, int i, float px, float py, float pz,
                                       float scene_bits, bool to_v2, bool rest, float4* xr) {
  if (to_v2) {
    const float rho = a.rho[i];
    xr[i] = make_float4(px, py, pz, (rho > 0.0f) ? (c.mass / rho) : 0.0f);
  }
  float4 x = a.x[i];
  float vx = (px - x.x) / c.dt;
  float vy = (py - x.y) / c.dt;
  float vz = (pz - x.z) / c.dt;
  x.x = px;
  x.y = py;
  x.z = pz;
  a.x[i] = x;
  if (rest && c.rest_on) restitution(c, px, py, pz, vx, vy, vz);
  (to_v2 ? a.v2 : a.v)[i] = make_float4(vx, vy, vz, scene_bits);
}

// The rest of a delta pass once the sums (ax, ay, az) of particle i are
// complete: scale by 1/rho0, plane projection (core.cpp:368-393), then the
// next iteration's p* or the commit.
__device__ __forceinline__ void delta_out(const StepArgs& a, const SceneConst& c, int i, const float4 p, float ax,
                                          float ay, float az, int in, int last, int to_v2, int rest,
                                          float4* q_out) {
  ax *= c.inv_density;
  ay *= c.inv_density;
  az *= c.inv_density;
  if (q_out) q_out[i] = make_float4(p.x + ax, p.y + ay, p.z + az, 0.0f);  // recorded for the adjoint
  if (c.plane_count > 0) {  // core.cpp:372-393
    float qx = p.x + ax, qy = p.y + ay, qz = p.z + az;
    for (int q = 0; q < c.plane_count; ++q) {
      const float4 pl = c.planes[q];
      const float sd = pl.x * qx + pl.y * qy + pl.z * qz - pl.w;
      const float pen = -sd;
      if (pen > 0.0f) {
        qx += pl.x * pen;
        qy += pl.y * pen;
        qz += pl.z * pen;
      }
    }
    ax = qx - p.x;
    ay = qy - p.y;
    az = qz - p.z;
  }
  const float nx = p.x + ax, ny = p.y + ay, nz = p.z + az;  // core.cpp:404-406
  if (!last) {
    a.p[in ^ 1][i] = make_float4(nx, ny, nz, p.w);
  } else {
    commit(a, c, i, nx, ny, nz, p.w, to_v2 != 0, rest != 0, a.p[in ^ 1]);
  }
}

// kPow: the s_corr exponent when every scene with s_corr shares it (2, 3,
// 4), else 0 (read per scene).
// kLiveIn: only the live ones among the first entries (live bits from the
// lambda pass of this iteration, same positions).
template <int U, int kPow, bool kLiveIn, bool kIeee = false>
__global__ void __launch_bounds__(kMaxBlock, FGB_LIST_MIN_BLOCKS) k_delta(StepArgs a, int in, int last, int to_v2, int rest, float4* q_out) {
  if (failed(a.status)) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const float4 p = a.p[in][i];
  const SceneConst& c = a.sc[__float_as_int(p.w)];
  const int n = a.cnt[i];
  const float4* __restrict__ pl = a.pl;  // {p_j, lambda_j} in one record
  const float li = a.lambda[i];
  const float h2 = c.h2;
  float ax = 0.0f, ay = 0.0f, az = 0.0f;
  const bool scorr = c.scorr_on != 0;
  auto one = [&](const float4 r) {
    const float dx = p.x - r.x, dy = p.y - r.y, dz = p.z - r.z;
    const float r2 = dist2(dx, dy, dz);
    if (r2 < h2) {
      const float gf = spiky(c, clamped_r<kIeee>(c, r2));
      float s = li + r.w;
      if (scorr) {
        const float ratio = poly6(c, r2) * c.scorr_inv_wdq;
        s += c.scorr_neg_k * pow_k<kPow>(ratio, c.scorr_n);
      }
      ax += s * gf * dx;
      ay += s * gf * dy;
      az += s * gf * dz;
    }
  };
  auto load = [&](int j) { return __ldg(pl + j); };
  const unsigned long long live =
      kLiveIn ? (static_cast<unsigned long long>(a.live[i]) | (static_cast<unsigned long long>(a.live[a.n + i]) << 32))
              : 0ull;
  const float4 dead = make_float4(INFINITY, p.y, p.z, 0.0f);
  with_list(a, i, [&](const auto& list) {
    if constexpr (U == 1) {
      if constexpr (kLiveIn) for_each_live_then<1>(list, n, live, load, dead, one, one);
      else for_each_neighbor<1>(list, n, load, one);
    } else {
      // Two entries at a time: the same operations as one() on a, then on b,
      // with the per-entry terms in paired arithmetic (pmul keeps each
      // product rounded on its own).
      const float2 px = f2(p.x), py = f2(p.y), pz = f2(p.z), nz = f2(c.neg_zero);
      auto two = [&](const float4 qa, const float4 qb) {
        const PairGeom g = pair_geom(px, py, pz, qa, qb, nz);
        const bool oka = g.r2.x < h2, okb = g.r2.y < h2;
        if (!oka && !okb) return;
        const float2 gf = spiky_pair<kIeee>(c, g.r2, nz);
        float2 s = padd(f2(li), make_float2(qa.w, qb.w));
        if (scorr) {
          const float2 ratio = pmul(poly6_pair(c, g.r2, nz), f2(c.scorr_inv_wdq), nz);
          float2 pw;
          if (kPow == 2) {
            pw = pmul(ratio, ratio, nz);
          } else if (kPow == 3) {
            pw = pmul(pmul(ratio, ratio, nz), ratio, nz);
          } else if (kPow == 4) {
            const float2 sq = pmul(ratio, ratio, nz);
            pw = pmul(sq, sq, nz);
          } else {
            pw = make_float2(pow_n(ratio.x, c.scorr_n), pow_n(ratio.y, c.scorr_n));
          }
          s = padd(s, pmul(f2(c.scorr_neg_k), pw, nz));
        }
        const float2 sg = pmul(s, gf, nz);
        const float2 tx = pmul(sg, g.dx, nz), ty = pmul(sg, g.dy, nz), tz = pmul(sg, g.dz, nz);
        if (oka) {
          ax += tx.x;
          ay += ty.x;
          az += tz.x;
        }
        if (okb) {
          ax += tx.y;
          ay += ty.y;
          az += tz.y;
        }
      };
      if constexpr (kLiveIn) for_each_live_then<U>(list, n, live, load, dead, two, one);
      else for_each_neighbor_pair<U>(list, n, load, two, one);
    }
  });
  delta_out(a, c, i, p, ax, ay, az, in, last, to_v2, rest, q_out);
}

// Commit without Jacobi iterations (solver_iterations == 0).
__global__ void __launch_bounds__(kMaxBlock) k_commit(StepArgs a, int to_v2, int rest) {
  if (failed(a.status)) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const float4 p = a.p[0][i];
  commit(a, a.sc[__float_as_int(p.w)], i, p.x, p.y, p.z, p.w, to_v2 != 0, rest != 0, a.p[1]);
}

// XSPH (core.cpp:423-466): reads v2 (committed) and the committing pass's
// {x, m / rho} records xr, writes v.
// kLiveOut: record the live bits of the committed positions for the
// vorticity passes (all ones where this scene skips XSPH).
template <int U, bool kLiveOut>
__global__ void __launch_bounds__(kMaxBlock, FGB_LIST_MIN_BLOCKS) k_xsph(StepArgs a, int rest, const float4* xr) {
  if (failed(a.status)) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const float4* __restrict__ xs = xr;
  const float4* __restrict__ vs = a.v2;
  const float4 xi = xs[i];
  const float4 vi = vs[i];
  const SceneConst& c = a.sc[__float_as_int(vi.w)];
  float vx = vi.x, vy = vi.y, vz = vi.z;
  unsigned long long bits = ~0ull;
  if (c.xsph_on) {
    const int n = a.cnt[i];
    const float h2 = c.h2;
    float sx = 0.0f, sy = 0.0f, sz = 0.0f;
    auto load = [&](int j) { return PosVel{__ldg(xs + j), __ldg(vs + j)}; };
    auto one = [&](const PosVel r) {
      const float r2 = dist2(xi.x - r.x.x, xi.y - r.x.y, xi.z - r.x.z);
      if (r2 < h2) {
        const float W = poly6(c, r2);
        const float inv_rho_j = r.x.w;
        sx += (r.v.x - vi.x) * W * inv_rho_j;
        sy += (r.v.y - vi.y) * W * inv_rho_j;
        sz += (r.v.z - vi.z) * W * inv_rho_j;
      }
      return r2 < h2;
    };
    with_list(a, i, [&](const auto& list) {
      if constexpr (U == 1) {
        if constexpr (kLiveOut) {
          bits = 0ull;
          int k = 0;
          for_each_neighbor<1>(list, n, load, [&](const PosVel r) {
            if (one(r) && k < kLiveEntries) bits |= 1ull << k;
            ++k;
          });
        } else {
          for_each_neighbor<1>(list, n, load, one);
        }
      } else {
        // Two entries at a time, as one() on a then on b (paired arithmetic).
        const float2 px = f2(xi.x), py = f2(xi.y), pz = f2(xi.z), nz = f2(c.neg_zero);
        auto two = [&](const PosVel ra, const PosVel rb) -> unsigned {
          const PairGeom g = pair_geom(px, py, pz, ra.x, rb.x, nz);
          const bool oka = g.r2.x < h2, okb = g.r2.y < h2;
          if (!oka && !okb) return 0u;
          const float2 w = poly6_pair(c, g.r2, nz);
          const float2 ir = make_float2(ra.x.w, rb.x.w);
          const float2 tx = pmul(pmul(psub(make_float2(ra.v.x, rb.v.x), f2(vi.x)), w, nz), ir, nz);
          const float2 ty = pmul(pmul(psub(make_float2(ra.v.y, rb.v.y), f2(vi.y)), w, nz), ir, nz);
          const float2 tz = pmul(pmul(psub(make_float2(ra.v.z, rb.v.z), f2(vi.z)), w, nz), ir, nz);
          if (oka) {
            sx += tx.x;
            sy += ty.x;
            sz += tz.x;
          }
          if (okb) {
            sx += tx.y;
            sy += ty.y;
            sz += tz.y;
          }
          return (oka ? 1u : 0u) | (okb ? 2u : 0u);
        };
        if constexpr (kLiveOut) bits = for_each_neighbor_pair_rec<U>(list, n, load, two, one);
        else for_each_neighbor_pair<U>(list, n, load, two, one);
      }
    });
    vx += c.visc_c * sx;
    vy += c.visc_c * sy;
    vz += c.visc_c * sz;
  }
  if (kLiveOut) store_live(a.live, a.n, i, bits);
  if (rest && c.rest_on) restitution(c, xi.x, xi.y, xi.z, vx, vy, vz);
  a.v[i] = make_float4(vx, vy, vz, vi.w);
}

// Vorticity omega and |omega| (core.cpp:472-508). kLive: 1 = only the live
// ones among the first entries (live bits from XSPH, same positions); 2 =
// record the live bits for the eta pass (no XSPH this step).
// Takes sqrtf for r in every scene (the same bits as rn_sqrt where that is
// checked): with rn_sqrt this pass ran 0.672 ms against 0.625 at the collapsed
// 125k step, the same at the 1M lattice step.
template <int U, int kLive>
__global__ void __launch_bounds__(kMaxBlock, FGB_LIST_MIN_BLOCKS) k_omega(StepArgs a) {
  if (failed(a.status)) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const float4* __restrict__ xs = a.x;
  const float4* __restrict__ vs = a.v;
  const float4 xi = xs[i];
  const float4 vi = vs[i];
  const SceneConst& c = a.sc[__float_as_int(vi.w)];
  float ox = 0.0f, oy = 0.0f, oz = 0.0f;
  unsigned long long bits = ~0ull;
  if (c.vort_on) {
    const int n = a.cnt[i];
    const float h2 = c.h2;
    auto load = [&](int j) { return PosVel{__ldg(xs + j), __ldg(vs + j)}; };
    auto one = [&](const PosVel r) {
      const float dx = xi.x - r.x.x, dy = xi.y - r.x.y, dz = xi.z - r.x.z;
      const float r2 = dist2(dx, dy, dz);
      if (r2 < h2) {
        const float gf = spiky(c, clamped_r<true>(c, r2));
        const float gx = gf * dx, gy = gf * dy, gz = gf * dz;
        const float ux = r.v.x - vi.x, uy = r.v.y - vi.y, uz = r.v.z - vi.z;
        ox += uy * gz - uz * gy;
        oy += uz * gx - ux * gz;
        oz += ux * gy - uy * gx;
      }
      return r2 < h2;
    };
    // Two entries at a time, as one() on a then on b (paired arithmetic).
    const float2 px = f2(xi.x), py = f2(xi.y), pz = f2(xi.z), nz = f2(c.neg_zero);
    auto two = [&](const PosVel ra, const PosVel rb) -> unsigned {
      const PairGeom g = pair_geom(px, py, pz, ra.x, rb.x, nz);
      const bool oka = g.r2.x < h2, okb = g.r2.y < h2;
      if (!oka && !okb) return 0u;
      const float2 gf = spiky_pair<true>(c, g.r2, nz);
      const float2 gx = pmul(gf, g.dx, nz), gy = pmul(gf, g.dy, nz), gz = pmul(gf, g.dz, nz);
      const float2 ux = psub(make_float2(ra.v.x, rb.v.x), f2(vi.x));
      const float2 uy = psub(make_float2(ra.v.y, rb.v.y), f2(vi.y));
      const float2 uz = psub(make_float2(ra.v.z, rb.v.z), f2(vi.z));
      const float2 cx = psub(pmul(uy, gz, nz), pmul(uz, gy, nz));
      const float2 cy = psub(pmul(uz, gx, nz), pmul(ux, gz, nz));
      const float2 cz = psub(pmul(ux, gy, nz), pmul(uy, gx, nz));
      if (oka) {
        ox += cx.x;
        oy += cy.x;
        oz += cz.x;
      }
      if (okb) {
        ox += cx.y;
        oy += cy.y;
        oz += cz.y;
      }
      return (oka ? 1u : 0u) | (okb ? 2u : 0u);
    };
    with_list(a, i, [&](const auto& list) {
      if constexpr (kLive == 1) {
        const PosVel dead{make_float4(INFINITY, xi.y, xi.z, 0.0f), make_float4(0.0f, 0.0f, 0.0f, 0.0f)};
        for_each_live_then<U>(list, n, static_cast<unsigned long long>(a.live[i]) |
                                           (static_cast<unsigned long long>(a.live[a.n + i]) << 32),
                              load, dead, two, one);
      } else if constexpr (U == 1) {
        bits = 0ull;
        int k = 0;
        for_each_neighbor<1>(list, n, load, [&](const PosVel r) {
          if (one(r) && k < kLiveEntries) bits |= 1ull << k;
          ++k;
        });
      } else {
        bits = for_each_neighbor_pair_rec<U>(list, n, load, two, one);
      }
    });
  }
  if (kLive == 2) store_live(a.live, a.n, i, bits);
  const float mag = sqrtf(ox * ox + oy * oy + oz * oz);
  a.omega[i] = make_float4(ox, oy, oz, mag);
  a.pl[i] = make_float4(xi.x, xi.y, xi.z, mag);  // the record k_eta gathers per neighbour
}

// Confinement force from eta = (ex, ey, ez) and omega oi, added to v
// (core.cpp:551-570).
__device__ __forceinline__ void confine(const SceneConst& c, const float4 oi, float ex, float ey, float ez, float4& v) {
  const float len = sqrtf(ex * ex + ey * ey + ez * ez);
  float nx = 0.0f, ny = 0.0f, nz2 = 0.0f;
  if (len > c.vort_norm_eps) {
    const float inv = 1.0f / len;
    nx = ex * inv;
    ny = ey * inv;
    nz2 = ez * inv;
  }
  const float fx = c.vort_eps * (ny * oi.z - nz2 * oi.y);
  const float fy = c.vort_eps * (nz2 * oi.x - nx * oi.z);
  const float fz = c.vort_eps * (nx * oi.y - ny * oi.x);
  v.x += c.dt * fx;
  v.y += c.dt * fy;
  v.z += c.dt * fz;
}

// Eta, confinement force, velocity update (core.cpp:512-570) and plane
// restitution (core.cpp:573-612); only the live ones among the first
// entries (live bits of these positions from XSPH or omega).
template <int U, bool kIeee = false>
__global__ void __launch_bounds__(kMaxBlock, FGB_LIST_MIN_BLOCKS) k_eta(StepArgs a, int rest) {
  if (failed(a.status)) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const float4* __restrict__ xo = a.pl;  // {x_j, |omega_j|}, written by k_omega
  const float4 xi = a.x[i];
  float4 v = a.v[i];
  const SceneConst& c = a.sc[__float_as_int(v.w)];
  if (c.vort_on) {
    const float4 oi = a.omega[i];
    const int n = a.cnt[i];
    const float h2 = c.h2;
    float ex = 0.0f, ey = 0.0f, ez = 0.0f;
    auto load = [&](int j) { return __ldg(xo + j); };
    auto one = [&](const float4 r) {
      const float dx = xi.x - r.x, dy = xi.y - r.y, dz = xi.z - r.z;
      const float r2 = dist2(dx, dy, dz);
      if (r2 < h2) {
        const float gf = spiky(c, clamped_r<kIeee>(c, r2));
        const float coeff = r.w - oi.w;
        ex += coeff * (gf * dx);
        ey += coeff * (gf * dy);
        ez += coeff * (gf * dz);
      }
    };
    // Two entries at a time, as one() on a then on b (paired arithmetic).
    const float2 px = f2(xi.x), py = f2(xi.y), pz = f2(xi.z), nz = f2(c.neg_zero);
    auto two = [&](const float4 ra, const float4 rb) {
      const PairGeom g = pair_geom(px, py, pz, ra, rb, nz);
      const bool oka = g.r2.x < h2, okb = g.r2.y < h2;
      if (!oka && !okb) return;
      const float2 gf = spiky_pair<kIeee>(c, g.r2, nz);
      const float2 coeff = psub(make_float2(ra.w, rb.w), f2(oi.w));
      const float2 tx = pmul(coeff, pmul(gf, g.dx, nz), nz);
      const float2 ty = pmul(coeff, pmul(gf, g.dy, nz), nz);
      const float2 tz = pmul(coeff, pmul(gf, g.dz, nz), nz);
      if (oka) {
        ex += tx.x;
        ey += ty.x;
        ez += tz.x;
      }
      if (okb) {
        ex += tx.y;
        ey += ty.y;
        ez += tz.y;
      }
    };
    const float4 dead = make_float4(INFINITY, xi.y, xi.z, 0.0f);
    with_list(a, i, [&](const auto& list) {
      for_each_live_then<U>(list, n, static_cast<unsigned long long>(a.live[i]) |
                                         (static_cast<unsigned long long>(a.live[a.n + i]) << 32),
                            load, dead, two, one);
    });
    confine(c, oi, ex, ey, ez, v);
  }
  if (rest && c.rest_on) restitution(c, xi.x, xi.y, xi.z, v.x, v.y, v.z);
  a.v[i] = v;
}

// ---------------------------------------------------------------------------
// Several lanes per particle.
//
// With G lanes per particle (G = 2, 4 or 8: a group of consecutive lanes of
// one warp, so a warp serves 32/G particles and a launch has G threads per
// particle), the lanes of a group split the particle's list into rounds: in
// round r lane u of the group takes entry rG + u, loads its index and record
// (the next round's record is loaded while this one is used) and computes the
// entry's terms with the same float operations as the one-lane walk. Then
// every lane of the group adds the round's G terms in list order, each moved
// by shuffle from the lane that computed it, so the sums are bit-identical to
// the one-lane walk's (an entry out of range or past the list's end adds
// nothing) and every lane of the group ends with them; the group's first
// lane writes the results.
//
// This takes a long list's dependent loads and term arithmetic off a single
// lane at the cost of the shuffles: it pays where a launch is short of warps
// (small scenes, or a collapsed scene whose launch fills less than a wave and
// lasts as long as its deepest lists) and loses in a launch that fills every
// SM, so the autotuner chooses G per kernel on the live state. Live bits are
// assembled from each round's ballot; passes that would read live bits walk
// every entry instead (a dead entry adds nothing).

// Thread -> (particle slot, lane within its group, group's first warp lane).
// Every lane of the warp takes part in the walk (a lane past the last
// particle, or of a scene that skips the pass, walks an empty list), so
// the shuffles and ballots run on the whole warp at once: shuffles whose masks
// named only a group would let the warp's groups run their rounds apart and
// serialise them.
template <int G>
struct LaneGroup {
  int i, sub, lead;
  __device__ __forceinline__ LaneGroup() {
    const long long t = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    i = static_cast<int>(t / G);
    const int lane = threadIdx.x & 31;
    sub = lane & (G - 1);
    lead = lane & ~(G - 1);
  }
  __device__ __forceinline__ float min_over(float v) const {
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(kFull, v, o));
    return v;
  }
};

// Terms of one list entry: K floats and whether the entry is within h.
template <int K>
struct Terms {
  float f[K];
  bool live;
  __device__ __forceinline__ Terms shfl(int src) const {
    Terms o;
#pragma unroll
    for (int q = 0; q < K; ++q) o.f[q] = __shfl_sync(kFull, f[q], src);
    o.live = false;
    return o;
  }
};

// Walks entries rG + sub (rounds r = 0, 1, ... up to the warp's longest
// list) of a list of n entries: term(record, in_list) gives an entry's Terms,
// add(Terms) accumulates, and each lane of the group adds the round's G terms
// in list order. Called by every lane of the warp. Returns the live bits of
// entries 0..63 (the same on every lane of the group).
template <int G, int K, typename LS, typename Load, typename Term, typename Add>
__device__ __forceinline__ unsigned long long walk_lanes(const LS& list, int n, const LaneGroup<G>& L,
                                                         Load&& load, Term&& term, Add&& add) {
  using Rec = decltype(load(0));
  unsigned long long bits = 0ull;
  const int rounds = __reduce_max_sync(kFull, (n + G - 1) / G);
  int k = L.sub;
  int j1 = (k + G < n) ? list.entry(k + G) : 0;
  Rec cur = (k < n) ? load(list.entry(k)) : Rec{};
  for (int r = 0; r < rounds; ++r, k += G) {
    const int j2 = (k + 2 * G < n) ? list.entry(k + 2 * G) : 0;
    if (k + kListAhead < n) prefetch_row(list.row(k + kListAhead));
    const Rec nxt = (k + G < n) ? load(j1) : Rec{};
    const Terms<K> t = term(cur, k < n);
    const unsigned lb = (__ballot_sync(kFull, t.live) >> L.lead) & ((1u << G) - 1u);
#pragma unroll
    for (int u = 0; u < G; ++u) {
      const Terms<K> tu = t.shfl(L.lead + u);
      if ((lb >> u) & 1u) add(tu);
    }
    if (r * G < kLiveEntries) bits |= static_cast<unsigned long long>(lb) << (r * G);
    cur = nxt;
    j1 = j2;
  }
  return bits;
}

template <int G, bool kLiveOut>
__global__ void __launch_bounds__(kMaxBlock, FGB_LIST_MIN_BLOCKS) k_lambda_lanes(StepArgs a, int in) {
  if (failed(a.status)) return;
  const LaneGroup<G> L;
  const int i = L.i;
  const bool valid = i < a.n;
  const float4* __restrict__ pos = a.p[in];
  const float4 p = valid ? pos[i] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  const int scene = valid ? __float_as_int(p.w) : 0;
  const SceneConst& c = a.sc[scene];
  const float h2 = c.h2;
  LambdaAcc acc;
  const int n = valid ? a.cnt[i] : 0;
  auto load = [&](int j) { return __ldg(pos + j); };
  auto term = [&](const float4 q, bool in_list) {  // LambdaAcc::add, term by term
    Terms<5> t;
    const float dx = p.x - q.x, dy = p.y - q.y, dz = p.z - q.z;
    const float r2 = dist2(dx, dy, dz);
    t.live = in_list && r2 < h2;
    if (t.live) {
      t.f[0] = poly6(c, r2);
      const float gf = spiky(c, clamped_r(c, r2));
      t.f[1] = gf * dx;
      t.f[2] = gf * dy;
      t.f[3] = gf * dz;
      const float ng = -c.grad_scale;
      const float jx = ng * t.f[1], jy = ng * t.f[2], jz = ng * t.f[3];
      t.f[4] = jx * jx + jy * jy + jz * jz;
    } else {
      t.f[0] = t.f[1] = t.f[2] = t.f[3] = t.f[4] = 0.0f;
    }
    return t;
  };
  auto add = [&](const Terms<5>& t) {
    acc.rho += t.f[0];
    acc.gsx += t.f[1];
    acc.gsy += t.f[2];
    acc.gsz += t.f[3];
    acc.sum_g2 += t.f[4];
  };
  unsigned long long bits = 0ull;
  with_list_lanes(a, i, valid, [&](const auto& list) { bits = walk_lanes<G, 5>(list, n, L, load, term, add); });
  if (!valid || L.sub != 0) return;
  if constexpr (kLiveOut) store_live(a.live, a.n, i, bits);
  float rho;
  const float lam = finish_lambda(c, acc.rho, acc.gsx, acc.gsy, acc.gsz, acc.sum_g2, rho);
  a.lambda[i] = lam;
  a.rho[i] = rho;
  a.pl[i] = make_float4(p.x, p.y, p.z, lam);
}

template <int G, int kPow, bool kLiveIn>
__global__ void __launch_bounds__(kMaxBlock, FGB_LIST_MIN_BLOCKS)
    k_delta_lanes(StepArgs a, int in, int last, int to_v2, int rest, float4* q_out) {
  if (failed(a.status)) return;
  const LaneGroup<G> L;
  const int i = L.i;
  const bool valid = i < a.n;
  const float4 p = valid ? a.p[in][i] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  const SceneConst& c = a.sc[valid ? __float_as_int(p.w) : 0];
  const float4* __restrict__ pl = a.pl;
  const float li = valid ? a.lambda[i] : 0.0f;
  const float h2 = c.h2;
  float ax = 0.0f, ay = 0.0f, az = 0.0f;
  const bool scorr = c.scorr_on != 0;
  const int n = valid ? a.cnt[i] : 0;
  auto load = [&](int j) { return __ldg(pl + j); };
  auto term = [&](const float4 r, bool in_list) {  // k_delta's one(), term by term
    Terms<3> t;
    const float dx = p.x - r.x, dy = p.y - r.y, dz = p.z - r.z;
    const float r2 = dist2(dx, dy, dz);
    t.live = in_list && r2 < h2;
    if (t.live) {
      const float gf = spiky(c, clamped_r(c, r2));
      float sc = li + r.w;
      if (scorr) {
        const float ratio = poly6(c, r2) * c.scorr_inv_wdq;
        sc += c.scorr_neg_k * pow_k<kPow>(ratio, c.scorr_n);
      }
      t.f[0] = sc * gf * dx;
      t.f[1] = sc * gf * dy;
      t.f[2] = sc * gf * dz;
    } else {
      t.f[0] = t.f[1] = t.f[2] = 0.0f;
    }
    return t;
  };
  auto add = [&](const Terms<3>& t) {
    ax += t.f[0];
    ay += t.f[1];
    az += t.f[2];
  };
  with_list_lanes(a, i, valid, [&](const auto& list) { walk_lanes<G, 3>(list, n, L, load, term, add); });
  if (!valid || L.sub != 0) return;
  delta_out(a, c, i, p, ax, ay, az, in, last, to_v2, rest, q_out);
}

template <int G, bool kLiveOut>
__global__ void __launch_bounds__(kMaxBlock, FGB_LIST_MIN_BLOCKS) k_xsph_lanes(StepArgs a, int rest, const float4* xr) {
  if (failed(a.status)) return;
  const LaneGroup<G> L;
  const int i = L.i;
  const bool valid = i < a.n;
  const float4* __restrict__ xs = xr;
  const float4* __restrict__ vs = a.v2;
  const float4 xi = valid ? xs[i] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  const float4 vi = valid ? vs[i] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  const int scene = valid ? __float_as_int(vi.w) : 0;
  const SceneConst& c = a.sc[scene];
  float vx = vi.x, vy = vi.y, vz = vi.z;
  const bool walk = valid && c.xsph_on;
  const int n = walk ? a.cnt[i] : 0;
  const float h2 = c.h2;
  float sx = 0.0f, sy = 0.0f, sz = 0.0f;
  auto load = [&](int j) { return PosVel{__ldg(xs + j), __ldg(vs + j)}; };
  auto term = [&](const PosVel r, bool in_list) {  // k_xsph's one(), term by term
    Terms<3> t;
    const float r2 = dist2(xi.x - r.x.x, xi.y - r.x.y, xi.z - r.x.z);
    t.live = in_list && r2 < h2;
    if (t.live) {
      const float W = poly6(c, r2);
      const float inv_rho_j = r.x.w;
      t.f[0] = (r.v.x - vi.x) * W * inv_rho_j;
      t.f[1] = (r.v.y - vi.y) * W * inv_rho_j;
      t.f[2] = (r.v.z - vi.z) * W * inv_rho_j;
    } else {
      t.f[0] = t.f[1] = t.f[2] = 0.0f;
    }
    return t;
  };
  auto add = [&](const Terms<3>& t) {
    sx += t.f[0];
    sy += t.f[1];
    sz += t.f[2];
  };
  unsigned long long bits = 0ull;
  with_list_lanes(a, i, valid, [&](const auto& list) { bits = walk_lanes<G, 3>(list, n, L, load, term, add); });
  if (!valid || L.sub != 0) return;
  if (c.xsph_on) {
    vx += c.visc_c * sx;
    vy += c.visc_c * sy;
    vz += c.visc_c * sz;
  } else {
    bits = ~0ull;  // no XSPH in this scene: the vorticity passes walk every entry
  }
  if (kLiveOut) store_live(a.live, a.n, i, bits);
  if (rest && c.rest_on) restitution(c, xi.x, xi.y, xi.z, vx, vy, vz);
  a.v[i] = make_float4(vx, vy, vz, vi.w);
}

// kLive: 1 = live bits given (unused: every entry is walked); 2 = record them.
template <int G, int kLive>
__global__ void __launch_bounds__(kMaxBlock, FGB_LIST_MIN_BLOCKS) k_omega_lanes(StepArgs a) {
  if (failed(a.status)) return;
  const LaneGroup<G> L;
  const int i = L.i;
  const bool valid = i < a.n;
  const float4* __restrict__ xs = a.x;
  const float4* __restrict__ vs = a.v;
  const float4 xi = valid ? xs[i] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  const float4 vi = valid ? vs[i] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  const SceneConst& c = a.sc[valid ? __float_as_int(vi.w) : 0];
  float ox = 0.0f, oy = 0.0f, oz = 0.0f;
  const int n = (valid && c.vort_on) ? a.cnt[i] : 0;
  const float h2 = c.h2;
  auto load = [&](int j) { return PosVel{__ldg(xs + j), __ldg(vs + j)}; };
  auto term = [&](const PosVel r, bool in_list) {  // k_omega's one(), term by term
    Terms<3> t;
    const float dx = xi.x - r.x.x, dy = xi.y - r.x.y, dz = xi.z - r.x.z;
    const float r2 = dist2(dx, dy, dz);
    t.live = in_list && r2 < h2;
    if (t.live) {
      const float gf = spiky(c, clamped_r<true>(c, r2));
      const float gx = gf * dx, gy = gf * dy, gz = gf * dz;
      const float ux = r.v.x - vi.x, uy = r.v.y - vi.y, uz = r.v.z - vi.z;
      t.f[0] = uy * gz - uz * gy;
      t.f[1] = uz * gx - ux * gz;
      t.f[2] = ux * gy - uy * gx;
    } else {
      t.f[0] = t.f[1] = t.f[2] = 0.0f;
    }
    return t;
  };
  auto add = [&](const Terms<3>& t) {
    ox += t.f[0];
    oy += t.f[1];
    oz += t.f[2];
  };
  unsigned long long bits = 0ull;
  with_list_lanes(a, i, valid, [&](const auto& list) { bits = walk_lanes<G, 3>(list, n, L, load, term, add); });
  if (!valid || L.sub != 0) return;
  if (!c.vort_on) bits = ~0ull;
  if (kLive == 2) store_live(a.live, a.n, i, bits);
  const float mag = sqrtf(ox * ox + oy * oy + oz * oz);
  a.omega[i] = make_float4(ox, oy, oz, mag);
  a.pl[i] = make_float4(xi.x, xi.y, xi.z, mag);
}

template <int G>
__global__ void __launch_bounds__(kMaxBlock, FGB_LIST_MIN_BLOCKS) k_eta_lanes(StepArgs a, int rest) {
  if (failed(a.status)) return;
  const LaneGroup<G> L;
  const int i = L.i;
  const bool valid = i < a.n;
  const float4* __restrict__ xo = a.pl;
  const float4 xi = valid ? a.x[i] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  float4 v = valid ? a.v[i] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  const SceneConst& c = a.sc[valid ? __float_as_int(v.w) : 0];
  const float4 oi = (valid && c.vort_on) ? a.omega[i] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  const int n = (valid && c.vort_on) ? a.cnt[i] : 0;
  const float h2 = c.h2;
  float ex = 0.0f, ey = 0.0f, ez = 0.0f;
  auto load = [&](int j) { return __ldg(xo + j); };
  auto term = [&](const float4 r, bool in_list) {  // k_eta's one(), term by term
    Terms<3> t;
    const float dx = xi.x - r.x, dy = xi.y - r.y, dz = xi.z - r.z;
    const float r2 = dist2(dx, dy, dz);
    t.live = in_list && r2 < h2;
    if (t.live) {
      const float gf = spiky(c, clamped_r(c, r2));
      const float coeff = r.w - oi.w;
      t.f[0] = coeff * (gf * dx);
      t.f[1] = coeff * (gf * dy);
      t.f[2] = coeff * (gf * dz);
    } else {
      t.f[0] = t.f[1] = t.f[2] = 0.0f;
    }
    return t;
  };
  auto add = [&](const Terms<3>& t) {
    ex += t.f[0];
    ey += t.f[1];
    ez += t.f[2];
  };
  with_list_lanes(a, i, valid, [&](const auto& list) { walk_lanes<G, 3>(list, n, L, load, term, add); });
  if (!valid || L.sub != 0) return;
  if (c.vort_on) confine(c, oi, ex, ey, ez, v);
  if (rest && c.rest_on) restitution(c, xi.x, xi.y, xi.z, v.x, v.y, v.z);
  a.v[i] = v;
}

// ---------------------------------------------------------------------------
// Upload / download / reset.

// Caller-order SoA arrays into slot-order x/v. With bmin (the stateless
// step over page-locked arrays, whose read of the host link bounds this
// kernel) it also adds each particle's predicted cell to the bounding box,
// the work of k_bounds, which that step's graph then leaves out.
__global__ void __launch_bounds__(kBlock) k_upload(const float* px, const float* py, const float* pz,
                                                   const float* vx, const float* vy, const float* vz,
                                                   float4* x, float4* v, int* slot, float* rho,
                                                   const SceneConst* sc, int scenes, int n, int* bmin, int* bmax) {
  const int o = blockIdx.x * kBlock + threadIdx.x;
  int scene = -1;
  int cx = 0, cy = 0, cz = 0;
  bool ok = false;
  if (o < n) {
    int lo = 0, hi = scenes - 1;  // last scene whose first slot <= o
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (sc[mid].first_slot <= o) lo = mid; else hi = mid - 1;
    }
    const float4 xo = make_float4(px[o], py[o], pz[o], __int_as_float(o));
    const float4 vo = make_float4(vx[o], vy[o], vz[o], __int_as_float(lo));
    x[o] = xo;
    v[o] = vo;
    slot[o] = o;
    rho[o] = 0.0f;
    if (bmin) {
      float4 vp = vo;
      scene = lo;
      ok = cell_of(sc[lo], predict(sc[lo], xo, vp), cx, cy, cz);
    }
  }
  if (bmin) add_bounds(bmin, bmax, scene, ok, cx, cy, cz);
}

__global__ void __launch_bounds__(kBlock) k_download(const float4* x, const float4* v, const int* slot,
                                                     float* px, float* py, float* pz, float* vx, float* vy,
                                                     float* vz, int n) {
  const int o = blockIdx.x * kBlock + threadIdx.x;
  if (o >= n) return;
  const int s = slot[o];
  const float4 xs = x[s];
  const float4 vs = v[s];
  px[o] = xs.x;
  py[o] = xs.y;
  pz[o] = xs.z;
  vx[o] = vs.x;
  vy[o] = vs.y;
  vz[o] = vs.z;
}

// One float4 field (x or v) of the step's output, caller order, into three
// arrays, targets[0..2]; nothing is written when the step failed. Any grid
// covers all n (grid-stride), so the write-out that runs beside the velocity
// passes can take a few blocks and leave the SMs to those passes.
__global__ void __launch_bounds__(kBlock) k_download_field(const float4* src, const int* slot,
                                                           float* const* targets, int n, const DevStatus* status) {
  if (failed(status)) return;
  for (int o = blockIdx.x * kBlock + threadIdx.x; o < n; o += gridDim.x * kBlock) {
    const float4 f = src[slot[o]];
    targets[0][o] = f.x;
    targets[1][o] = f.y;
    targets[2][o] = f.z;
  }
}

__global__ void k_reset(DevStatus* st, int* bmin, int* bmax, int scenes) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t == 0) {
    st->err = 0;
    st->started = 0;
    st->step = 0;
    st->fail_step = 0;
    st->need_grid = 0;
    st->need_nbr = 0;
  }
  for (int k = t; k < 3 * scenes; k += gridDim.x * blockDim.x) {
    bmin[k] = INT_MAX;
    bmax[k] = INT_MIN;
  }
}

inline int blocks_for(long long n, int threads) { return static_cast<int>((n + threads - 1) / threads); }


// Blocks of a list pass with `lanes` threads per particle.
inline int list_grid(const StepArgs& a, int block, int lanes) {
  return blocks_for(static_cast<long long>(a.n) * lanes, block);
}

// Launch shape of list kernel k in the plan: block size, records fetched
// ahead (one lane per particle) and lanes per particle.
// A list pass's launch shape. ieee: some scene's clamped r^2 range lies
// outside rn_sqrt's checked range, so lambda, delta and eta run their
// one-lane, four-ahead form with sqrtf (any shape gives the same bits; the
// vorticity pass takes sqrtf in every form).
struct ListShape {
  int block, unroll, lanes;
  bool ieee;
  ListShape(const StepPlan& plan, int k)
      : block(plan.block[k]), unroll(plan.unroll[k]), lanes(plan.lanes[k]), ieee(plan.ieee_sqrt) {}
};

template <int kPow, bool kLiveIn>
struct DeltaPow {
  template <int U>
  static void launch(int block, cudaStream_t st, const StepArgs& a, int in, int last, int to_v2, int rest,
                     float4* q_out) {
    k_delta<U, kPow, kLiveIn><<<list_grid(a, block, 1), block, 0, st>>>(a, in, last, to_v2, rest, q_out);
  }
  template <int G>
  static void launch_lanes(int block, cudaStream_t st, const StepArgs& a, int in, int last, int to_v2, int rest,
                           float4* q_out) {
    k_delta_lanes<G, kPow, kLiveIn><<<list_grid(a, block, G), block, 0, st>>>(a, in, last, to_v2, rest, q_out);
  }
  static void dispatch(const ListShape& sh, cudaStream_t st, const StepArgs& a, int in, int last, int to_v2,
                       int rest, float4* q_out) {
    const int b = sh.block;
    if (sh.ieee) {
      k_delta<4, kPow, kLiveIn, true><<<list_grid(a, b, 1), b, 0, st>>>(a, in, last, to_v2, rest, q_out);
      return;
    }
    switch (sh.lanes) {
      case 2: launch_lanes<2>(b, st, a, in, last, to_v2, rest, q_out); return;
      case 4: launch_lanes<4>(b, st, a, in, last, to_v2, rest, q_out); return;
      case 8: launch_lanes<8>(b, st, a, in, last, to_v2, rest, q_out); return;
      default: break;
    }
    switch (sh.unroll) {
      case 1: launch<1>(b, st, a, in, last, to_v2, rest, q_out); break;
      case 2: launch<2>(b, st, a, in, last, to_v2, rest, q_out); break;
      case 8: launch<8>(b, st, a, in, last, to_v2, rest, q_out); break;
      default: launch<4>(b, st, a, in, last, to_v2, rest, q_out); break;
    }
  }
};

template <bool kLiveIn>
void launch_delta_pow(const StepPlan& plan, cudaStream_t st, const StepArgs& a, int in, int last, int to_v2, int rest,
                      float4* q_out) {
  const ListShape sh(plan, FLUID_KERNEL_DELTA);
  switch (plan.scorr_pow) {
    case 2: DeltaPow<2, kLiveIn>::dispatch(sh, st, a, in, last, to_v2, rest, q_out); break;
    case 3: DeltaPow<3, kLiveIn>::dispatch(sh, st, a, in, last, to_v2, rest, q_out); break;
    case 4: DeltaPow<4, kLiveIn>::dispatch(sh, st, a, in, last, to_v2, rest, q_out); break;
    default: DeltaPow<0, kLiveIn>::dispatch(sh, st, a, in, last, to_v2, rest, q_out); break;
  }
}

// live: the lambda pass of this iteration recorded live bits (iterations
// after the first).
void launch_delta(const StepPlan& plan, cudaStream_t st, const StepArgs& a, int in, int last, int to_v2, int rest,
                  float4* q_out, bool live) {
  if (live) launch_delta_pow<true>(plan, st, a, in, last, to_v2, rest, q_out);
  else launch_delta_pow<false>(plan, st, a, in, last, to_v2, rest, q_out);
}

template <bool kLiveOut>
void launch_lambda(const StepPlan& plan, cudaStream_t st, const StepArgs& a, int in) {
  const ListShape sh(plan, FLUID_KERNEL_LAMBDA);
  const int b = sh.block;
  if (sh.ieee) {
    k_lambda<4, kLiveOut, true><<<list_grid(a, b, 1), b, 0, st>>>(a, in);
    return;
  }
  switch (sh.lanes) {
    case 2: k_lambda_lanes<2, kLiveOut><<<list_grid(a, b, 2), b, 0, st>>>(a, in); return;
    case 4: k_lambda_lanes<4, kLiveOut><<<list_grid(a, b, 4), b, 0, st>>>(a, in); return;
    case 8: k_lambda_lanes<8, kLiveOut><<<list_grid(a, b, 8), b, 0, st>>>(a, in); return;
    default: break;
  }
  const int g = list_grid(a, b, 1);
  switch (sh.unroll) {
    case 1: k_lambda<1, kLiveOut><<<g, b, 0, st>>>(a, in); break;
    case 2: k_lambda<2, kLiveOut><<<g, b, 0, st>>>(a, in); break;
    case 8: k_lambda<8, kLiveOut><<<g, b, 0, st>>>(a, in); break;
    default: k_lambda<4, kLiveOut><<<g, b, 0, st>>>(a, in); break;
  }
}

template <bool kLiveOut>
void launch_xsph(const StepPlan& plan, cudaStream_t st, const StepArgs& a, int rest, const float4* xr) {
  const ListShape sh(plan, FLUID_KERNEL_XSPH);
  const int b = sh.block;
  switch (sh.lanes) {
    case 2: k_xsph_lanes<2, kLiveOut><<<list_grid(a, b, 2), b, 0, st>>>(a, rest, xr); return;
    case 4: k_xsph_lanes<4, kLiveOut><<<list_grid(a, b, 4), b, 0, st>>>(a, rest, xr); return;
    case 8: k_xsph_lanes<8, kLiveOut><<<list_grid(a, b, 8), b, 0, st>>>(a, rest, xr); return;
    default: break;
  }
  const int g = list_grid(a, b, 1);
  switch (sh.unroll) {
    case 1: k_xsph<1, kLiveOut><<<g, b, 0, st>>>(a, rest, xr); break;
    case 2: k_xsph<2, kLiveOut><<<g, b, 0, st>>>(a, rest, xr); break;
    case 8: k_xsph<8, kLiveOut><<<g, b, 0, st>>>(a, rest, xr); break;
    default: k_xsph<4, kLiveOut><<<g, b, 0, st>>>(a, rest, xr); break;
  }
}

template <int kLive>
void launch_omega(const StepPlan& plan, cudaStream_t st, const StepArgs& a) {
  const ListShape sh(plan, FLUID_KERNEL_OMEGA);
  const int b = sh.block;
  switch (sh.lanes) {
    case 2: k_omega_lanes<2, kLive><<<list_grid(a, b, 2), b, 0, st>>>(a); return;
    case 4: k_omega_lanes<4, kLive><<<list_grid(a, b, 4), b, 0, st>>>(a); return;
    case 8: k_omega_lanes<8, kLive><<<list_grid(a, b, 8), b, 0, st>>>(a); return;
    default: break;
  }
  const int g = list_grid(a, b, 1);
  switch (sh.unroll) {
    case 1: k_omega<1, kLive><<<g, b, 0, st>>>(a); break;
    case 2: k_omega<2, kLive><<<g, b, 0, st>>>(a); break;
    case 8: k_omega<8, kLive><<<g, b, 0, st>>>(a); break;
    default: k_omega<4, kLive><<<g, b, 0, st>>>(a); break;
  }
}

void launch_eta(const StepPlan& plan, cudaStream_t st, const StepArgs& a, int rest) {
  const ListShape sh(plan, FLUID_KERNEL_ETA);
  const int b = sh.block;
  if (sh.ieee) {
    k_eta<4, true><<<list_grid(a, b, 1), b, 0, st>>>(a, rest);
    return;
  }
  switch (sh.lanes) {
    case 2: k_eta_lanes<2><<<list_grid(a, b, 2), b, 0, st>>>(a, rest); return;
    case 4: k_eta_lanes<4><<<list_grid(a, b, 4), b, 0, st>>>(a, rest); return;
    case 8: k_eta_lanes<8><<<list_grid(a, b, 8), b, 0, st>>>(a, rest); return;
    default: break;
  }
  const int g = list_grid(a, b, 1);
  switch (sh.unroll) {
    case 1: k_eta<1><<<g, b, 0, st>>>(a, rest); break;
    case 2: k_eta<2><<<g, b, 0, st>>>(a, rest); break;
    case 8: k_eta<8><<<g, b, 0, st>>>(a, rest); break;
    default: k_eta<4><<<g, b, 0, st>>>(a, rest); break;
  }
}

// The cell-key sort at one digit width: digit counts, then `passes` passes
// (those beyond the step's own pass count return at entry).
template <int kBits>
void launch_sort(const StepArgs& a, int passes, cudaStream_t st, LaunchMarks& m) {
  const int digit_blocks = a.tiles < kRadixDigitBlocks ? a.tiles : kRadixDigitBlocks;
  k_radix_digits<kBits><<<digit_blocks, kBlock, 0, st>>>(a);
  m.mark(FLUID_KERNEL_RADIX_HIST);
  for (int pass = 0; pass < passes; ++pass) {
    k_radix_onesweep<kBits><<<a.tiles, sort_threads(kBits), 0, st>>>(a, pass);
    m.mark(FLUID_KERNEL_RADIX_SCATTER);
  }
}

}  // namespace

void LaunchMarks::start() {
  next = 0;
  if (!on) return;
  if (capturing) {
    cudaEventRecordWithFlags((*events)[0], stream, cudaEventRecordExternal);
  } else {
    cudaEventRecord((*events)[0], stream);
  }
  next = 1;
}

void LaunchMarks::mark(int stage) {
  ++launches;
  if (!on) return;
  if (next >= static_cast<int>(events->size())) return;
  (*stages)[next] = stage;
  if (capturing) {
    cudaEventRecordWithFlags((*events)[next], stream, cudaEventRecordExternal);
  } else {
    cudaEventRecord((*events)[next], stream);
  }
  ++next;
}

cudaError_t enqueue_step(const StepArgs& args, const StepPlan& plan, cudaStream_t st, LaunchMarks& m,
                         const StepRecord* rec, const StepDownload* dl) {
  StepArgs a = args;
  if (rec) a.list16 = 0;  // the adjoint reads the recorded lists as 32-bit rows
  const int nb = blocks_for(a.n, kBlock);
  m.start();
  if (!(dl && dl->bounds_done)) {
    k_bounds<<<nb, kBlock, 0, st>>>(a);
    m.mark(FLUID_KERNEL_BOUNDS);
  }
  k_grid_setup<<<1, kBlock, 0, st>>>(a, plan.radix_bits);
  m.mark(FLUID_KERNEL_GRID);
  k_keys<<<nb, kBlock, 0, st>>>(a);
  m.mark(FLUID_KERNEL_KEYS);
  if (a.n <= kRadixTile) {  // one tile: the whole sort in one block
    k_radix_tile<<<1, kBlock, 0, st>>>(a);
    m.mark(FLUID_KERNEL_RADIX_SCATTER);
  } else {
    switch (plan.radix_bits) {
      case 11: launch_sort<11>(a, plan.radix_passes, st, m); break;
      case 9: launch_sort<9>(a, plan.radix_passes, st, m); break;
      default: launch_sort<8>(a, plan.radix_passes, st, m); break;
    }
  }
  k_reorder<<<nb, kBlock, 0, st>>>(a);
  m.mark(FLUID_KERNEL_REORDER);
  const size_t n4 = sizeof(float4) * static_cast<size_t>(a.n);
  const size_t n1 = sizeof(float) * static_cast<size_t>(a.n);
  if (rec) {
    cudaMemcpyAsync(rec->x0, a.x, n4, cudaMemcpyDeviceToDevice, st);
    cudaMemcpyAsync(rec->p, a.p[0], n4, cudaMemcpyDeviceToDevice, st);
  }
  const int bc = plan.block[FLUID_KERNEL_NBR_BUILD] > kMaxBuildBlock ? kMaxBuildBlock : plan.block[FLUID_KERNEL_NBR_BUILD];
  a.stage_rows = plan.stage_rows;
  const size_t stage_bytes = sizeof(int) * (plan.stage_rows + 1) * bc;
  if (plan.stage_rows == kStageRowsDefault) k_nbr_build<kStageRowsDefault><<<blocks_for(a.n, bc), bc, stage_bytes, st>>>(a);
  else k_nbr_build<0><<<blocks_for(a.n, bc), bc, stage_bytes, st>>>(a);
  m.mark(FLUID_KERNEL_NBR_BUILD);

  const bool post = plan.xsph || plan.vorticity;
  const int to_v2 = plan.xsph ? 1 : 0;
  const int rest_commit = (!post && plan.restitution) ? 1 : 0;
  if (plan.iterations == 0) {
    k_commit<<<nb, kBlock, 0, st>>>(a, to_v2, rest_commit);
    m.mark(FLUID_KERNEL_COMMIT);
  }
  for (int it = 0; it < plan.iterations; ++it) {
    const int in = it & 1;
    {
      if (it == 0) launch_lambda<false>(plan, st, a, in);
      else launch_lambda<true>(plan, st, a, in);
      m.mark(FLUID_KERNEL_LAMBDA);
      if (rec)
        cudaMemcpyAsync(rec->lambda + static_cast<size_t>(it) * a.n, a.lambda, n1, cudaMemcpyDeviceToDevice, st);
    }
    const int last = (it == plan.iterations - 1) ? 1 : 0;
    float4* q_out = rec ? rec->q + static_cast<size_t>(it) * a.n : nullptr;
    launch_delta(plan, st, a, in, last, to_v2, last ? rest_commit : 0, q_out, it > 0);
    m.mark(FLUID_KERNEL_DELTA);
    if (rec)  // p^(it+1); the last iteration's lands in x (commit)
      cudaMemcpyAsync(rec->p + static_cast<size_t>(it + 1) * a.n, last ? a.x : a.p[in ^ 1], n4,
                      cudaMemcpyDeviceToDevice, st);
  }
  if (rec) cudaMemcpyAsync(rec->rho, a.rho, n1, cudaMemcpyDeviceToDevice, st);
  if (dl) {  // positions are final: write them out beside the velocity passes
    cudaEventRecord(dl->committed, st);
    cudaStreamWaitEvent(dl->aux, dl->committed, 0);
    const int bx = (dl->blocks > 0 && dl->blocks < nb) ? dl->blocks : nb;
    k_download_field<<<bx, kBlock, 0, dl->aux>>>(a.x, a.slot, dl->targets, a.n, a.status);
    cudaEventRecord(dl->positions_done, dl->aux);
  }
  if (plan.xsph) {
    // The committing pass left {x, m / rho} in the p buffer it did not use.
    const float4* xr = a.p[plan.iterations == 0 ? 1 : (plan.iterations & 1)];
    const int rest = (!plan.vorticity && plan.restitution) ? 1 : 0;
    if (plan.vorticity) launch_xsph<true>(plan, st, a, rest, xr);
    else launch_xsph<false>(plan, st, a, rest, xr);
    m.mark(FLUID_KERNEL_XSPH);
  }
  if (plan.vorticity) {
    // Live bits of the committed positions: from XSPH when it ran, else
    // recorded here; the eta pass reads them.
    if (plan.xsph) launch_omega<1>(plan, st, a);
    else launch_omega<2>(plan, st, a);
    m.mark(FLUID_KERNEL_OMEGA);
    if (rec && rec->omega) cudaMemcpyAsync(rec->omega, a.omega, n4, cudaMemcpyDeviceToDevice, st);
    launch_eta(plan, st, a, plan.restitution ? 1 : 0);
    m.mark(FLUID_KERNEL_ETA);
  }
  if (dl) {
    k_download_field<<<nb, kBlock, 0, st>>>(a.v, a.slot, dl->targets + 3, a.n, a.status);
    cudaStreamWaitEvent(st, dl->positions_done, 0);
  }
  return cudaGetLastError();
}

cudaError_t enqueue_upload(const float* px, const float* py, const float* pz, const float* vx, const float* vy,
                           const float* vz, float4* x, float4* v, int* slot, float* rho, const SceneConst* sc,
                           int scenes, int n, cudaStream_t st, int* bmin, int* bmax) {
  if (n > 0)
    k_upload<<<blocks_for(n, kBlock), kBlock, 0, st>>>(px, py, pz, vx, vy, vz, x, v, slot, rho, sc, scenes, n, bmin,
                                                       bmax);
  return cudaGetLastError();
}

cudaError_t enqueue_download(const float4* x, const float4* v, const int* slot, float* px, float* py, float* pz,
                             float* vx, float* vy, float* vz, int n, cudaStream_t st) {
  if (n > 0) k_download<<<blocks_for(n, kBlock), kBlock, 0, st>>>(x, v, slot, px, py, pz, vx, vy, vz, n);
  return cudaGetLastError();
}

cudaError_t enqueue_reset(DevStatus* status, int* bmin, int* bmax, int scenes, cudaStream_t st) {
  k_reset<<<1, kBlock, 0, st>>>(status, bmin, bmax, scenes);
  return cudaGetLastError();
}

}  // namespace fgb
