// Shared device-side types of the GB300 PBF timestep.
//
// Layout in HBM (one solver, all scenes back to back, N particles):
//   x[2], v[2]    float4 per slot, cell-sorted order of the current step;
//                 x.w = caller index (int bits), v.w = scene (int bits).
//                 Parity buffers: a step reads [p] and writes [1-p], so a
//                 step that has to be re-run still has its input.
//   slot[2]       int per caller index: its slot in x/v.
//   p0, p1        float4 predicted positions (p.w = scene), ping-pong over
//                 the Jacobi iterations.
//   v2            float4 velocity scratch for XSPH; omega float4 (w = |omega|).
//   pl            float4 {p.xyz, lambda} of the current Jacobi iteration, so
//                 the delta pass gathers one record per neighbour.
//   lambda, rho[2] float per slot.
//   keys/vals     radix-sort ping-pong (u32 cell key, int caller index).
//   table         int2 (first, end) per cell of the per-scene bounding grids.
//   cnt, nbr      neighbour lists in 32-wide slices: warp w (slots 32w..32w+31)
//                 owns depth[w] rows from wbase[w] (claimed by one atomic per
//                 block), entry k of lane l in row k, column l, so every
//                 list read is one coalesced access per warp. A row is 32
//                 ints, or 32 16-bit offsets from the warp's anchor (32w -
//                 32768) when slice_fmt[w] has kSlice16: the warps whose
//                 lists fit the shared-memory staging and whose entries all
//                 lie within 32768 slots of that anchor (the lattice phase;
//                 half the bytes for every pass to read).
#pragma once

#include <cstdint>

#include "fluid_gb300.h"
#include "pbf_sqrt.cuh"

namespace fgb {

constexpr int kBlock = 256;
constexpr int kRadixItems = 16;                     // keys per thread of the 256-thread sort kernels
constexpr int kRadixTile = kBlock * kRadixItems;    // keys per CTA
// k_radix_onesweep's block at a digit width: 512 threads (8 keys each) up to
// 9-bit digits; 256 at 11 bits, where 16 warps' digit counts would not fit
// in static shared memory.
constexpr int sort_threads(int bits) { return bits <= 9 ? 512 : 256; }
constexpr int kRadixMaxBins = 1 << 11;                // widest digit (11 bits)
constexpr int kRadixMaxPasses = 4;                  // passes of a u32 key at 8-bit digits
constexpr int kRadixDigitBlocks = 304;              // k_radix_digits grid (stride over tiles)
constexpr unsigned kFull = 0xffffffffu;

// Per-scene constants, each computed on the host with the same float
// operations, in the same order, as the reference computes it
// (core/src/core.cpp:138-148, 270-274 and the kernel helpers :35-71).
struct SceneConst {
  float h, inv_h, h2, min_r2;
  float poly6_c;     // 315 / (64 pi h^9)
  float w0;          // W(0) = poly6_c * h2^3
  float spiky_c;     // -45 / (pi h^6)
  float mass, inv_density, grad_scale, epsilon, density;
  float scorr_inv_wdq, scorr_neg_k;
  int scorr_n, scorr_on;
  float dt, gdt_x, gdt_y, gdt_z;  // external force * dt
  float visc_c;
  int xsph_on;
  float vort_eps, vort_norm_eps;
  int vort_on;
  float rest_neg_e;               // -restitution
  int rest_on;
  int plane_count;
  int iterations;
  int all_pairs;                  // use_uniform_grid == 0: lists from all pairs
  int first_slot, count;          // particle range of the scene
  float neg_zero;                 // -0.0f, read at run time (see pmul in the kernels)
  int exact_sqrt;                 // 1: clamped r^2 range outside rn_sqrt's checked range (the plan then uses sqrtf)
  float4 planes[FLUID_MAX_PLANES];  // (nx, ny, nz, d)
  float rest_scale[FLUID_MAX_PLANES];  // 1 - friction of each plane
};

// Bounding grid of one scene for the current step.
struct GridInfo {
  int minx, miny, minz;
  int dimx, dimy, dimz;
  uint32_t base;  // first key of the scene
  int pad;
};

// Device status word. Kernels read `err` on entry and return when set, so
// after a failure the rest of the enqueued work is a no-op and the failed
// step's input buffers stay intact.
struct DevStatus {
  int err;        // fluid_status of the first failure
  int started;    // steps started in this batch
  int step;       // index within the batch of the step in progress
  int fail_step;  // step index within the batch that failed
  int npass;      // radix passes needed this step
  unsigned epoch; // steps started on this status word (never reset): tags the sort's look-back words
  unsigned long long total_cells;
  unsigned long long need_grid;
  unsigned long long need_nbr;
  unsigned long long pairs;  // sum of neighbour counts, this step
  unsigned long long cursor; // list entries claimed by the slices, this step
  int nbr_max;
  int pad;
};

// Every pointer one step needs, parity already resolved.
struct StepArgs {
  const float4* x_old;
  const float4* v_old;
  const int* slot_old;
  const float* rho_old;
  float4* x;
  float4* v;
  float4* v2;
  int* slot;
  float4* p[2];
  float4* omega;
  float4* pl;              // {p.xyz, lambda}, written by the lambda pass
  uint32_t* live;          // 2 x n: live bits of each list's first 64 entries at one set of positions
  float* lambda;
  float* rho;
  uint32_t* keys[2];
  int* vals[2];
  unsigned long long* look;  // tiles x (1 << radix bits) look-back words of the sort pass
  int* radix_next;           // kRadixMaxPasses tile counters of the sort passes
  uint32_t* digit_total;     // kRadixMaxPasses x kRadixMaxBins: counts, then starts
  int2* table;
  int* cnt;
  int* depth;             // per warp
  long long* wbase;       // per warp
  int* slice_fmt;         // per warp: slice format, kSliceOverflow | kSlice16 bits
  int* nbr;
  int* bmin;              // 3 per scene
  int* bmax;
  GridInfo* grid;
  DevStatus* status;
  const SceneConst* sc;
  int n;
  int scenes;
  int tiles;              // radix tiles
  int warps;              // ceil(n / 32)
  long long grid_capacity;
  long long nbr_capacity;
  int list16;             // 1: the list build may store 16-bit slices (0 for steps recorded for the adjoint)
  int stage_rows;         // list entries per lane the build stages in shared memory
};

// Slice format bits (StepArgs::slice_fmt, per warp).
constexpr int kSliceOverflow = 1;  // longer than the staging: the build's second scan wrote the entries past it
constexpr int kSlice16 = 2;        // 16-bit offsets from the warp's anchor
constexpr int kSliceAnchorBack = 32768;  // anchor of warp w: 32 w - 32768

}  // namespace fgb
