/*
 * fluid_gb300.h — C ABI of the GB300 (sm_103a) Position Based Fluids timestep.
 *
 * This is the drop-in boundary for the CUDA backend of CTKnight/FluidSimulator.
 * Every entry point names the reference interface it replaces (path:line within
 * the reference project). All pointers are plain host or device pointers, all
 * sizes are element counts, and every call returns a fluid_status code; no C++
 * or torch types cross this boundary.
 *
 * Particle order at the boundary is always the caller's (original) order. The
 * solver keeps particles sorted by grid cell on the device and undoes that
 * permutation on download.
 *
 * Threading: a fluid_solver is single-threaded state; calls on one solver must
 * not overlap. Different solvers may be used from different threads.
 */
#ifndef FLUID_GB300_H
#define FLUID_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* 2: per-plane friction at the end of fluid_params. 3: entry points added
 * (fluid_solver_get/set_lanes, fluid_fill_block, fluid_fill_shape); every
 * struct is as in version 2. */
#define FLUID_GB300_ABI_VERSION 3
/* Planes per scene. The reference keeps an unbounded std::vector SoA
 * (core/include/fluid/core.h:44-78); every reference scene uses 6. */
#define FLUID_MAX_PLANES 32

typedef enum fluid_status {
  FLUID_OK = 0,
  FLUID_ERR_INVALID_ARGUMENT = 1, /* bad pointer, size or parameter */
  FLUID_ERR_CUDA = 2,             /* a CUDA runtime call failed */
  FLUID_ERR_CAPACITY = 3,         /* a device buffer could not grow enough */
  FLUID_ERR_DOMAIN = 4,           /* grid over the particles' cells too large */
  FLUID_ERR_NONFINITE = 5,        /* a predicted position was NaN or Inf */
  FLUID_ERR_NO_DEVICE = 6,        /* no CUDA device */
  FLUID_ERR_OUT_OF_MEMORY = 7,    /* device allocation failed */
  FLUID_ERR_NOT_SUPPORTED = 8,    /* parameter combination not implemented */
  FLUID_ERR_STATE = 9             /* call out of order (e.g. step before upload) */
} fluid_status;

/*
 * Mirrors fluid::Params (core/include/fluid/core.h:11-79) field for field, same
 * meaning and units. The plane SoA (core.h:44-78) becomes fixed arrays plus a
 * count so the struct holds no pointers. Params::backend (core.h:13-17) is not
 * carried: neither reference step function reads it. The last two fields
 * (per-plane friction) extend it; left zero they change nothing.
 */
typedef struct fluid_params {
  float dt;                      /* core.h:12 */
  float density;                 /* core.h:18, rest density rho0 */
  float particle_mass;           /* core.h:20 */
  float h;                       /* core.h:22, kernel radius = grid cell size */
  float particle_radius;         /* core.h:23, unused by the step */
  float epsilon;                 /* core.h:24, lambda relaxation */
  int32_t solver_iterations;     /* core.h:25 */
  float neighbor_reserve_factor; /* core.h:26, neighbour-list growth factor */
  int32_t use_uniform_grid;      /* core.h:27; 0 = all-pairs lists (O(N^2)) */
  int32_t enable_scorr;          /* core.h:28 */
  int32_t enable_xsph;           /* core.h:29 */
  int32_t enable_vorticity;      /* core.h:30 */
  float scorr_k;                 /* core.h:31 */
  int32_t scorr_n;               /* core.h:32 */
  float scorr_dq_coeff;          /* core.h:33 */
  float visc_c;                  /* core.h:34, XSPH c */
  float plane_restitution;       /* core.h:35 */
  float plane_friction;          /* core.h:36 */
  float vort_epsilon;            /* core.h:37 */
  float vort_norm_eps;           /* core.h:38 */
  float external_force[3];       /* core.h:39-43 */
  int32_t plane_count;           /* core.h:50 PlaneSoA::size() */
  float plane_nx[FLUID_MAX_PLANES];
  float plane_ny[FLUID_MAX_PLANES];
  float plane_nz[FLUID_MAX_PLANES];
  float plane_d[FLUID_MAX_PLANES]; /* signed distance = n.x - d */
  /* Per-plane friction, an extension with no fluid::Params counterpart: the
   * reference scene files give each collision plane a "friction" value that
   * its loader drops (core/src/init.cpp:371-414). When nonzero, plane q scales
   * the tangential velocity by 1 - plane_friction_each[q] in place of
   * 1 - plane_friction, and the contact pass runs when plane_restitution > 0
   * or any plane's friction > 0. Zero (the default) keeps the reference's
   * single friction. */
  int32_t plane_friction_per_plane;
  float plane_friction_each[FLUID_MAX_PLANES];
} fluid_params;

/* Fills *p with the defaults of core/include/fluid/core.h:12-43 (no planes). */
void fluid_params_default(fluid_params* p);

/* Replaces fluid::cuda_version (cuda/include/fluid/cuda.h:7). */
int fluid_gb300_version(void);

/*
 * Replaces fluid::cuda_device_available (cuda/include/fluid/cuda.h:8,
 * cuda/src/cuda_stub.cu:740-762). Returns 1 when at least one device is
 * present, else 0. *count receives the device count (0 on error); *error
 * receives a static message or NULL. Either pointer may be NULL.
 */
int fluid_gb300_device_available(int* count, const char** error);

/*
 * Replaces fluid::cuda_step(const Params&, State&) (cuda/include/fluid/cuda.h:9,
 * cuda/src/cuda_stub.cu:764-1099). Host SoA arrays of `count` particles in the
 * caller's order are advanced by one timestep in place and *time += dt, exactly
 * as the reference does. count == 0 only advances time (cuda_stub.cu:766-769).
 * Device buffers are cached per calling thread between calls (keyed by count),
 * so repeated calls allocate nothing; state still round-trips through the host
 * arrays every call, like the reference.
 */
int fluid_gb300_cuda_step(const fluid_params* params, int64_t count,
                          float* pos_x, float* pos_y, float* pos_z,
                          float* vel_x, float* vel_y, float* vel_z,
                          float* time);

/*
 * No counterpart in the reference: one timestep that allocates no device
 * memory, for callers that cannot allocate where they step the fluid (an
 * application that owns all device memory through its own pool or budget,
 * a frame-time loop where an allocation would stall, a plugin that must not
 * grow the process's footprint). The six arrays are the caller's DEVICE
 * arrays of `count` particles in caller order, advanced in place; *time +=
 * dt. Work is enqueued on `stream` (a cudaStream_t, NULL = legacy default)
 * and the call blocks until it is done: it synchronises `stream` once to
 * read the step's status and once after writing the arrays.
 *
 * All scratch lives in one fixed device array inside this library (about
 * 7.6 MiB, held on every GPU that loads the library until the process
 * exits). Limits: count <= FLUID_NOALLOC_MAX_PARTICLES, at most
 * FLUID_NOALLOC_MAX_NEIGHBOR_SLOTS neighbour-list entries (32-wide slices)
 * and FLUID_NOALLOC_MAX_CELLS grid cells per step; beyond any of them the
 * call returns FLUID_ERR_CAPACITY and leaves the arrays untouched. Every call
 * shares that scratch, so calls whose work overlaps on the GPU race: do not
 * run two at once. The first call on a device looks up the scratch address
 * on that device; make that first call before any stream capture.
 */
#define FLUID_NOALLOC_MAX_PARTICLES 8192
#define FLUID_NOALLOC_MAX_NEIGHBOR_SLOTS (1 << 20)
#define FLUID_NOALLOC_MAX_CELLS (1 << 18)
int fluid_gb300_step_noalloc(const fluid_params* params, int64_t count,
                             float* pos_x, float* pos_y, float* pos_z,
                             float* vel_x, float* vel_y, float* vel_z,
                             float* time, void* stream);

/* ---- Scene fills generated on the device ------------------------------- */

enum { FLUID_SHAPE_CUBE = 0, FLUID_SHAPE_SPHERE = 1 };

/*
 * init_block (core/src/init.cpp:72-106) written straight into the caller's
 * DEVICE arrays: particle (z * ny + y) * nx + x at origin + float(i) *
 * spacing per axis, the reference's order and float arithmetic. With jitter
 * > 0 each coordinate then gets + U(-jitter, jitter) from SplitMix64(seed)
 * draw 3m + axis + 1 (m = first + particle index), rounded to float and added
 * in float -- the seeded jitter of this project's benchmark scenes, so a
 * device-filled scene equals the host-filled one bit for bit. The arrays hold
 * nx * ny * nz floats. Synchronises `stream` before returning.
 */
int fluid_fill_block(int64_t nx, int64_t ny, int64_t nz, float origin_x,
                     float origin_y, float origin_z, float spacing,
                     double jitter, uint64_t seed, int64_t first,
                     float* pos_x, float* pos_y, float* pos_z, void* stream);

/*
 * One "shape" of a scene file (core/src/init.cpp:285-345): kind
 * FLUID_SHAPE_CUBE fills origin + spacing/2 + k * spacing below origin +
 * extent[d] on each axis; FLUID_SHAPE_SPHERE fills the cube around origin of
 * half-width extent[0] (the radius) and keeps the points with (dx*dx + dy*dy)
 * + dz*dz < r*r. Axes are accumulated in float as the reference's loops do,
 * points are in its loop order (x outermost, z innermost), velocities are
 * `velocity` (NULL = zero). Writes *count; when it exceeds `capacity`,
 * returns FLUID_ERR_CAPACITY without writing (call again with capacity >=
 * *count). Allocates a little device memory for the axes for the call.
 */
int fluid_fill_shape(int32_t kind, const float origin[3], const float extent[3],
                     float spacing, const float velocity[3], float* pos_x,
                     float* pos_y, float* pos_z, float* vel_x, float* vel_y,
                     float* vel_z, int64_t capacity, int64_t* count,
                     void* stream);

/* ---- Device-resident solver (no reference counterpart: the reference keeps
 * no device state between steps; this is the handle the drop-in above uses). */

typedef struct fluid_solver fluid_solver;

enum { FLUID_MEMORY_HOST = 0, FLUID_MEMORY_DEVICE = 1 };

/* Creates a solver on CUDA device `device` with its own non-blocking stream. */
int fluid_solver_create(fluid_solver** out, int device);
void fluid_solver_destroy(fluid_solver* solver);

/* Runs all later work on `stream` (a cudaStream_t); NULL restores the solver's own. */
int fluid_solver_set_stream(fluid_solver* solver, void* stream);

/*
 * Declares the scenes: `scene_count` independent scenes with params[s] and
 * counts[s] particles each. Particle arrays at the boundary hold the scenes
 * back to back (scene 0 first). A single simulation is scene_count == 1.
 * All scenes must share solver_iterations, the three enable_* flags and
 * use_uniform_grid; h, mass, planes and the rest may differ per scene.
 * Resets the time of every scene to 0 and drops any uploaded state.
 */
int fluid_solver_configure(fluid_solver* solver, int32_t scene_count,
                           const fluid_params* params, const int64_t* counts);

/* Replaces the parameters of the configured scenes without touching state. */
int fluid_solver_set_params(fluid_solver* solver, const fluid_params* params);

/* Copies state in (caller order). memory selects host or device pointers. */
int fluid_solver_upload(fluid_solver* solver,
                        const float* pos_x, const float* pos_y, const float* pos_z,
                        const float* vel_x, const float* vel_y, const float* vel_z,
                        int32_t memory);

/* Copies state out in caller order; synchronous. */
int fluid_solver_download(fluid_solver* solver,
                          float* pos_x, float* pos_y, float* pos_z,
                          float* vel_x, float* vel_y, float* vel_z,
                          int32_t memory);

/*
 * Advances every scene by `nsteps` timesteps and waits for the result. When a
 * step needs a larger neighbour list or cell table than is allocated, the step
 * is detected on the device, the buffers grow (by neighbor_reserve_factor, as
 * core/src/core.cpp:128-136 reserves), and that step is re-run from its own
 * untouched input, so results never depend on capacity.
 */
int fluid_solver_step(fluid_solver* solver, int32_t nsteps);

/* Enqueues `nsteps` timesteps without waiting. */
int fluid_solver_step_async(fluid_solver* solver, int32_t nsteps);

/* Waits for enqueued steps, re-running any that overflowed a capacity. */
int fluid_solver_synchronize(fluid_solver* solver);

/* Capture each timestep as a CUDA graph (1) or launch kernels directly (0). */
int fluid_solver_set_graphs(fluid_solver* solver, int32_t enable);

/* Records a CUDA event after every kernel of each step (adds no
 * synchronisation). Times accumulate at fluid_solver_synchronize for the
 * last completed step of each parity, i.e. for every step when the caller
 * synchronises after each step. */
int fluid_solver_set_profiling(fluid_solver* solver, int32_t enable);

/* Kernels of one step, in launch order (per-kernel timing buckets). */
enum {
  FLUID_KERNEL_BOUNDS = 0,   /* predicted cells, per-scene bounding box */
  FLUID_KERNEL_GRID = 1,     /* per-scene grid over the box */
  FLUID_KERNEL_KEYS = 2,     /* linear cell keys */
  FLUID_KERNEL_RADIX_HIST = 3,    /* sort: digit counts of every pass, one read */
  FLUID_KERNEL_RADIX_SCAN = 4,    /* no launches: the digit starts are found by
                                     each pass's look-back; id kept so the
                                     others keep their values */
  FLUID_KERNEL_RADIX_SCATTER = 5, /* sort: one pass per digit (rank, look-back, scatter) */
  FLUID_KERNEL_REORDER = 6,  /* gather into cell order + cell table */
  FLUID_KERNEL_NBR_BUILD = 7, /* lists (one scan) + slices */
  FLUID_KERNEL_NBR_OVERFLOW = 8, /* no launches: the list build writes long lists'
                                    remaining entries itself (second scan) */
  FLUID_KERNEL_LAMBDA = 9,
  FLUID_KERNEL_DELTA = 10,   /* position correction (+ commit on the last) */
  FLUID_KERNEL_COMMIT = 11,  /* commit when solver_iterations == 0 */
  FLUID_KERNEL_XSPH = 12,
  FLUID_KERNEL_OMEGA = 13,
  FLUID_KERNEL_ETA = 14,     /* eta + confinement + plane restitution */
  FLUID_KERNEL_COUNT = 15
};

/* Name of a kernel id ("k_delta", ...); NULL when out of range. */
const char* fluid_kernel_name(int kernel);

/* Sums of per-kernel GPU time (ms) and launch counts since the last reset,
 * indexed by FLUID_KERNEL_*. */
int fluid_solver_kernel_times(fluid_solver* solver, double* ms_out,
                              int64_t* launches_out, int32_t kernels,
                              int32_t reset);

/*
 * Autotuner (no reference counterpart). Times each tunable kernel (the
 * neighbour-list passes and the list build) under every launch shape --
 * neighbour entries fetched ahead in {2, 4, 8}, threads per block in
 * {128, 256, 512}, and for the list passes 2, 4 or 8 lanes per particle at
 * each block size -- over `trials` discarded steps of the current state. It
 * keeps each kernel's default shape (4 ahead; 128 threads for the list
 * passes, 256 for the build; the default lanes below) unless another is at
 * least 2 % faster, and else the fastest, per kernel. It then times the cell-key sort with 8-,
 * 9- and 11-bit digits and keeps the fastest width. One entry ahead (the
 * single-entry walker) is left out of the sweep: where all lists are short
 * it can win narrowly and then lose by far once they grow; set it with
 * fluid_solver_set_tuning. The state and time are not advanced. Every choice
 * computes identical results; only speed differs.
 */
int fluid_solver_autotune(fluid_solver* solver, int32_t trials);

/* Launch shape per kernel id (FLUID_KERNEL_*): entries fetched ahead and
 * threads per block. Arrays of `kernels` entries; either may be NULL. */
int fluid_solver_get_tuning(fluid_solver* solver, int32_t* unroll, int32_t* block,
                            int32_t kernels);
int fluid_solver_set_tuning(fluid_solver* solver, const int32_t* unroll,
                            const int32_t* block, int32_t kernels);

/* Lanes per particle of each neighbour-list pass (FLUID_KERNEL_LAMBDA, _DELTA,
 * _XSPH, _OMEGA, _ETA): 1 (one lane walks a particle's list; the unroll of
 * fluid_solver_set_tuning applies), or 2, 4 or 8 lanes that split the list
 * into rounds and add the round's terms in list order, for launches short of
 * warps. Every other kernel takes 1. By default lambda and delta take 8
 * when the solver's scenes hold at most 16,384 particles in all, 4 up to
 * 32,768, and 1 above; the other list passes take 1. The autotuner chooses it with the other
 * shapes; results are identical under every choice. (No counterpart in the
 * reference, whose CUDA step maps one thread to a particle.) */
int fluid_solver_get_lanes(fluid_solver* solver, int32_t* lanes, int32_t kernels);
int fluid_solver_set_lanes(fluid_solver* solver, const int32_t* lanes, int32_t kernels);

/* Digit width of the cell-key radix sort: 8, 9 (default) or 11 bits. Keys of
 * b bits take ceil(b / width) passes; the permutation does not depend on it. */
int fluid_solver_get_sort_bits(fluid_solver* solver, int32_t* bits);
int fluid_solver_set_sort_bits(fluid_solver* solver, int32_t bits);

/*
 * Reverse-mode derivative (no reference counterpart: the reference has no
 * adjoint). Cotangent arrays hold 3 * particles floats in caller order: all
 * x, then all y, then all z. Neighbour sets and every branch (r < h, the
 * 0.01 h clamp, plane contacts, restitution's vn < 0) are held at the forward
 * step's values, and so is the |eta| > vort_norm_eps test of vorticity
 * confinement.
 *
 * fluid_solver_step_backward: vector-Jacobian product of the step the current
 * state would take: given dL/d(positions, velocities) after that step, writes
 * dL/d(positions, velocities) of the current state and dL/d(visc_c) per scene
 * (g_visc_c, scene_count floats, may be NULL). The state, time and step
 * count are unchanged; the step is recomputed internally.
 */
int fluid_solver_step_backward(fluid_solver* solver, const float* g_pos_out,
                               const float* g_vel_out, float* g_pos_in,
                               float* g_vel_in, float* g_visc_c, int32_t memory);

/* Runs nsteps forward from the current state keeping a state snapshot every
 * checkpoint_every steps (for fluid_solver_backward); leaves the final state. */
int fluid_solver_record(fluid_solver* solver, int32_t nsteps, int32_t checkpoint_every);

/* Back-propagates dL/d(final state) of the last record() to dL/d(the state
 * record() started from) and dL/d(visc_c): each checkpoint segment is
 * recomputed forward, then stepped back in reverse. Leaves the final state. */
int fluid_solver_backward(fluid_solver* solver, const float* g_pos_final,
                          const float* g_vel_final, float* g_pos_initial,
                          float* g_vel_initial, float* g_visc_c, int32_t memory);

/* Time of scene `scene` (float, accumulated as State::time, core.cpp:614). */
int fluid_solver_get_time(fluid_solver* solver, int32_t scene, float* time);
int fluid_solver_set_time(fluid_solver* solver, int32_t scene, float time);

typedef struct fluid_stats {
  int64_t particles;
  int64_t steps;             /* completed steps since configure */
  int64_t neighbor_pairs;    /* directed pairs in the last step's lists */
  int32_t neighbor_max;      /* largest per-particle count, last step */
  int32_t grid_cells;        /* cells in the last step's bounding grids */
  int64_t neighbor_capacity; /* allocated list slots */
  int64_t grid_capacity;     /* allocated cell-table entries */
  int64_t regrows;           /* steps re-run after a capacity grew */
  int64_t kernel_launches;   /* kernels launched since configure */
} fluid_stats;

int fluid_solver_get_stats(fluid_solver* solver, fluid_stats* out);

/* Per-particle records of the last completed step, caller order. */
enum {
  FLUID_DEBUG_CELL_KEYS = 0,    /* int32 x3: floor(p* / h) per axis (core.cpp:28-34) */
  FLUID_DEBUG_SORTED_ORDER = 1, /* int32: caller index at each sorted position
                                   (core.cpp:173-183); per-scene local indices */
  FLUID_DEBUG_NEIGHBOR_COUNTS = 2, /* int32 (core.cpp:245-246 differences) */
  FLUID_DEBUG_RHO = 3,          /* float, last lambda pass (core.cpp:321) */
  FLUID_DEBUG_LAMBDA = 4        /* float, last lambda pass (core.cpp:328) */
};

/* Copies a debug record to host memory of `capacity` elements (int32/float). */
int fluid_solver_read_debug(fluid_solver* solver, int32_t what, void* host_out,
                            int64_t capacity);

/*
 * Frame output (replaces the reference's per-frame host read of State plus
 * VtkWriter::write_frame, app/src/main.cpp:259-274, io/src/vtk_writer.cpp).
 *
 * fluid_solver_frame_begin starts copying the current positions (and
 * velocities when host_vel is not NULL) into caller-owned host buffers of
 * 3 * particles floats (x block, y block, z block, caller order) -- pinned
 * memory makes the copy asynchronous. It waits for steps already enqueued,
 * then returns at once; the copy runs on its own stream and overlaps steps
 * enqueued afterwards. Two slots (0, 1) may be in flight; reusing a slot
 * waits for its previous copy. fluid_solver_frame_wait blocks until the
 * slot's copy has landed.
 */
int fluid_solver_frame_begin(fluid_solver* solver, int32_t slot, float* host_pos,
                             float* host_vel);
int fluid_solver_frame_wait(fluid_solver* solver, int32_t slot);

/* Writes one frame as VTK PolyData: binary == 0 reproduces the reference's
 * ASCII .vtp byte for byte (io/src/vtk_writer.cpp:25-79); binary != 0 writes
 * an appended raw block (20 bytes per particle). */
int fluid_write_vtp(const char* path, const float* pos_x, const float* pos_y,
                    const float* pos_z, int64_t count, int32_t binary);

/* Writes a ParaView collection of frames (io/src/vtk_writer.cpp:107-130). */
int fluid_write_pvd(const char* path, const double* times, const char* const* files,
                    int64_t count);

/* Last error message of this solver (static storage owned by the solver). */
const char* fluid_solver_last_error(const fluid_solver* solver);

/* Message for a status code. */
const char* fluid_status_string(int status);

#ifdef __cplusplus
}  /* extern "C" */
#endif

#endif /* FLUID_GB300_H */
