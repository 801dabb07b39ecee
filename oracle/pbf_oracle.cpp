// ORACLE — test infrastructure, not product code.
//
// A CPU restatement of the reference Position Based Fluids timestep
// (CTKnight/FluidSimulator core/src/core.cpp:119-615), templated on the
// arithmetic type. T = float is the checker the GPU path is compared against
// (bit-exact with the reference when both are compiled with -ffp-contract=off);
// T = double is the FP64 run used to report each path's error. Only the tests,
// the smoke check and the bench's CPU-baseline leg load this library; the
// product never links or calls it.
//
// Per-step scratch (neighbour list, rho, lambda, ...) lives in a workspace that
// persists across steps, as fluid::CpuScratch does inside fluid::State
// (core/include/fluid/core.h:81-132): with solver_iterations == 0 the XSPH pass
// reads the previous step's rho, exactly like the reference.

#include "fluid_gb300.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

template <typename T>
struct Pi;
template <>
struct Pi<float> {
  static constexpr float value = 3.14159265358979323846f;  // core.cpp:10
};
template <>
struct Pi<double> {
  static constexpr double value = 3.14159265358979323846;
};

// core.cpp:35-46
template <typename T>
T poly6(T r2, T h) {
  const T h2 = h * h;
  if (r2 > h2) return T(0);
  const T diff = h2 - r2;
  const T diff3 = diff * diff * diff;
  const T h4 = h2 * h2;
  const T h9 = h4 * h4 * h;
  const T coeff = T(315) / (T(64) * Pi<T>::value * h9);
  return coeff * diff3;
}

// core.cpp:48-57
template <typename T>
T spiky_factor(T r, T h) {
  if (r > h) return T(0);
  const T h2 = h * h;
  const T h6 = h2 * h2 * h2;
  const T diff = h - r;
  const T coeff = T(-45) / (Pi<T>::value * h6);
  return coeff * diff * diff;
}

// core.cpp:59-71
template <typename T>
T pow_n(T ratio, int n) {
  if (n == 2) return ratio * ratio;
  if (n == 3) return ratio * ratio * ratio;
  if (n == 4) {
    const T r2 = ratio * ratio;
    return r2 * r2;
  }
  return std::pow(ratio, static_cast<T>(n));
}

// Friction of plane q: the scene's single value (core.cpp:575), or the
// plane's own under the per-plane extension of fluid_params.
inline float plane_mu(const fluid_params& p, int q) {
  return p.plane_friction_per_plane ? p.plane_friction_each[q] : p.plane_friction;
}

// core.cpp:573-574: the contact pass runs when restitution or friction is on.
inline bool contacts_on(const fluid_params& p) {
  bool friction = false;
  for (int q = 0; q < p.plane_count; ++q) friction |= plane_mu(p, q) > 0.0f;
  return (p.plane_restitution > 0.0f || friction) && p.plane_count > 0;
}

struct Cell {
  int x, y, z;
};

inline bool cell_less(const Cell& a, const Cell& b) {  // core.cpp:12-21
  if (a.x != b.x) return a.x < b.x;
  if (a.y != b.y) return a.y < b.y;
  return a.z < b.z;
}
inline bool cell_eq(const Cell& a, const Cell& b) {  // core.cpp:23-26
  return a.x == b.x && a.y == b.y && a.z == b.z;
}

// core.cpp:28-34: floor(p * (1/h)), the multiply by the rounded reciprocal.
template <typename T>
Cell cell_of(T x, T y, T z, T cell) {
  const T inv = T(1) / cell;
  return Cell{static_cast<int>(std::floor(x * inv)),
              static_cast<int>(std::floor(y * inv)),
              static_cast<int>(std::floor(z * inv))};
}

template <typename T>
struct Workspace {
  std::vector<T> px, py, pz;        // predicted positions p*
  std::vector<T> dx, dy, dz;        // Jacobi corrections
  std::vector<T> lambda, rho;
  std::vector<T> dvx, dvy, dvz;     // XSPH
  std::vector<T> ox, oy, oz, omag;  // vorticity omega, |omega|
  std::vector<T> ex, ey, ez;        // eta
  std::vector<Cell> key;            // cell of p* per particle
  std::vector<int> order;           // particle at each sorted position
  std::vector<Cell> run_key;        // occupied cells, ascending
  std::vector<int> run_begin, run_end;
  std::vector<int> nbr;             // neighbour lists, back to back
  std::vector<int64_t> nbr_begin;   // count + 1 offsets into nbr

  void resize(std::size_t n) {
    for (auto* v : {&px, &py, &pz, &dx, &dy, &dz, &lambda, &rho, &dvx, &dvy,
                    &dvz, &ox, &oy, &oz, &omag, &ex, &ey, &ez}) {
      v->resize(n, T(0));
    }
    key.resize(n);
    order.resize(n);
    nbr_begin.resize(n + 1, 0);
  }
};

template <typename T>
struct Consts {
  T dt, h, h2, min_r2, inv_density, mass, grad_scale, epsilon;
  bool scorr;
  T scorr_inv_wdq, scorr_k;
  int scorr_n;
};

template <typename T>
Consts<T> make_consts(const fluid_params& p) {
  Consts<T> c{};
  c.dt = T(p.dt);
  c.h = T(p.h);
  c.h2 = c.h * c.h;
  const T min_r = T(0.01f) * c.h;  // core.cpp:141-142
  c.min_r2 = min_r * min_r;
  c.scorr = p.enable_scorr && p.scorr_k != 0.0f;  // core.cpp:143-148
  const T dq_coeff = (p.scorr_dq_coeff > 0.0f) ? T(p.scorr_dq_coeff) : T(0.3f);
  const T dq = dq_coeff * c.h;
  const T wdq = c.scorr ? poly6<T>(dq * dq, c.h) : T(0);
  c.scorr_inv_wdq = (wdq > T(1e-12f)) ? (T(1) / wdq) : T(0);
  c.scorr_k = T(p.scorr_k);
  c.scorr_n = p.scorr_n;
  c.inv_density = T(1) / T(p.density);  // core.cpp:270-274
  c.mass = T(p.particle_mass);
  c.grad_scale = c.mass * c.inv_density;
  c.epsilon = T(p.epsilon);
  return c;
}

// Neighbour lists from p* on the uniform grid (core.cpp:163-247): cells of
// size h, particles sorted by (cell x, y, z, index), each particle scanning the
// 27 cells in dz, dy, dx order and keeping j != i with r^2 < h^2 in scan order.
template <typename T>
void build_grid_lists(Workspace<T>& w, std::size_t n, T h, T h2) {
  for (std::size_t i = 0; i < n; ++i) {
    w.key[i] = cell_of(w.px[i], w.py[i], w.pz[i], h);
    w.order[i] = static_cast<int>(i);
  }
  std::sort(w.order.begin(), w.order.end(), [&](int a, int b) {
    if (cell_less(w.key[a], w.key[b])) return true;
    if (cell_less(w.key[b], w.key[a])) return false;
    return a < b;
  });
  w.run_key.clear();
  w.run_begin.clear();
  w.run_end.clear();
  for (std::size_t s = 0; s < n; ++s) {
    const Cell& k = w.key[w.order[s]];
    if (s == 0 || !cell_eq(k, w.run_key.back())) {
      if (s != 0) w.run_end.push_back(static_cast<int>(s));
      w.run_key.push_back(k);
      w.run_begin.push_back(static_cast<int>(s));
    }
  }
  w.run_end.push_back(static_cast<int>(n));

  w.nbr.clear();
  w.nbr_begin[0] = 0;
  for (std::size_t i = 0; i < n; ++i) {
    const T xi = w.px[i], yi = w.py[i], zi = w.pz[i];
    const Cell base = cell_of(xi, yi, zi, h);
    for (int oz = -1; oz <= 1; ++oz) {
      for (int oy = -1; oy <= 1; ++oy) {
        for (int ox = -1; ox <= 1; ++ox) {
          const Cell want{base.x + ox, base.y + oy, base.z + oz};
          auto it = std::lower_bound(w.run_key.begin(), w.run_key.end(), want,
                                     cell_less);
          if (it == w.run_key.end() || !cell_eq(*it, want)) continue;
          const std::size_t r = static_cast<std::size_t>(it - w.run_key.begin());
          for (int s = w.run_begin[r]; s < w.run_end[r]; ++s) {
            const int j = w.order[s];
            if (j == static_cast<int>(i)) continue;
            const T ddx = xi - w.px[j];
            const T ddy = yi - w.py[j];
            const T ddz = zi - w.pz[j];
            const T r2 = ddx * ddx + ddy * ddy + ddz * ddz;
            if (r2 < h2) w.nbr.push_back(j);
          }
        }
      }
    }
    w.nbr_begin[i + 1] = static_cast<int64_t>(w.nbr.size());
  }
}

// All-pairs lists in ascending j (core.cpp:248-268), for use_uniform_grid == 0.
template <typename T>
void build_pair_lists(Workspace<T>& w, std::size_t n, T h2) {
  w.nbr.clear();
  w.nbr_begin[0] = 0;
  for (std::size_t i = 0; i < n; ++i) {
    for (std::size_t j = 0; j < n; ++j) {
      if (i == j) continue;
      const T ddx = w.px[i] - w.px[j];
      const T ddy = w.py[i] - w.py[j];
      const T ddz = w.pz[i] - w.pz[j];
      const T r2 = ddx * ddx + ddy * ddy + ddz * ddz;
      if (r2 < h2) w.nbr.push_back(static_cast<int>(j));
    }
    w.nbr_begin[i + 1] = static_cast<int64_t>(w.nbr.size());
  }
}

// Forward internals of one step, for the adjoint (SoA blocks: x | y | z).
template <typename T>
struct Record {
  std::size_t n = 0;
  int iters = 0;
  bool vorticity = false;
  std::vector<T> x0, x1, v2, rho;          // input x, committed x, committed v, last rho
  std::vector<T> v3, om, omag;             // velocity after XSPH, omega (3n), |omega| (n)
  std::vector<std::vector<T>> P, Q, LAM;   // p^k (iters+1), pre-projection q^k (iters), lambda^k (iters)
  std::vector<int> nbr;
  std::vector<int64_t> nbr_begin;
};

template <typename T>
void put3(std::vector<T>& dst, std::size_t n, const T* a, const T* b, const T* c) {
  dst.resize(3 * n);
  std::copy(a, a + n, dst.begin());
  std::copy(b, b + n, dst.begin() + n);
  std::copy(c, c + n, dst.begin() + 2 * n);
}

template <typename T>
struct Dump {
  int32_t* cell_keys;
  int32_t* sorted_order;
  int32_t* neighbor_counts;
  T* rho;
  T* lambda;
};

template <typename T>
int step(Workspace<T>& w, const fluid_params& p, std::size_t n, T* X, T* Y,
         T* Z, T* VX, T* VY, T* VZ, T* time, const Dump<T>* dump,
         int64_t* pairs_out, int32_t* max_out, Record<T>* rec = nullptr) {
  w.resize(n);
  if (n == 0) {  // core.cpp:122-125
    *time += T(p.dt);
    return 0;
  }
  const Consts<T> c = make_consts<T>(p);
  const T h = c.h, h2 = c.h2, dt = c.dt;
  const T fx = T(p.external_force[0]), fy = T(p.external_force[1]),
          fz = T(p.external_force[2]);
  const long long N = static_cast<long long>(n);

  if (rec) {
    rec->n = n;
    rec->iters = p.solver_iterations;
    rec->vorticity = p.enable_vorticity && p.vort_epsilon != 0.0f;
    put3(rec->x0, n, X, Y, Z);
    rec->P.assign(p.solver_iterations + 1, {});
    rec->Q.assign(p.solver_iterations, std::vector<T>(3 * n));
    rec->LAM.assign(p.solver_iterations, {});
  }

  // Predict (core.cpp:150-161).
#pragma omp parallel for
  for (long long i = 0; i < N; ++i) {
    VX[i] += fx * dt;
    VY[i] += fy * dt;
    VZ[i] += fz * dt;
    w.px[i] = X[i] + VX[i] * dt;
    w.py[i] = Y[i] + VY[i] * dt;
    w.pz[i] = Z[i] + VZ[i] * dt;
  }

  const bool grid = p.use_uniform_grid && h > T(0);
  if (grid) {
    build_grid_lists(w, n, h, h2);
  } else {
    build_pair_lists(w, n, h2);
  }
  if (rec) {
    put3(rec->P[0], n, w.px.data(), w.py.data(), w.pz.data());
    rec->nbr = w.nbr;
    rec->nbr_begin = w.nbr_begin;
  }

  // Jacobi iterations (core.cpp:276-408).
  for (int iter = 0; iter < p.solver_iterations; ++iter) {
    // Density constraint and lambda (core.cpp:281-329).
#pragma omp parallel for
    for (long long i = 0; i < N; ++i) {
      const T xi = w.px[i], yi = w.py[i], zi = w.pz[i];
      T rho = T(0), gsx = T(0), gsy = T(0), gsz = T(0), sum_g2 = T(0);
      for (int64_t k = w.nbr_begin[i]; k < w.nbr_begin[i + 1]; ++k) {
        const int j = w.nbr[k];
        const T ddx = xi - w.px[j];
        const T ddy = yi - w.py[j];
        const T ddz = zi - w.pz[j];
        const T r2 = ddx * ddx + ddy * ddy + ddz * ddz;
        rho += poly6<T>(r2, h);
        if (r2 < h2) {
          const T r = std::sqrt(r2 < c.min_r2 ? c.min_r2 : r2);
          const T gf = spiky_factor<T>(r, h);
          const T gx = gf * ddx, gy = gf * ddy, gz = gf * ddz;
          gsx += gx;
          gsy += gy;
          gsz += gz;
          const T jx = -c.grad_scale * gx;
          const T jy = -c.grad_scale * gy;
          const T jz = -c.grad_scale * gz;
          sum_g2 += jx * jx + jy * jy + jz * jz;
        }
      }
      rho += poly6<T>(T(0), h);
      rho *= c.mass;
      w.rho[i] = rho;
      const T C = rho * c.inv_density - T(1);
      const T ix = c.grad_scale * gsx;
      const T iy = c.grad_scale * gsy;
      const T iz = c.grad_scale * gsz;
      sum_g2 += ix * ix + iy * iy + iz * iz;
      w.lambda[i] = -C / (sum_g2 + c.epsilon);
    }
    if (rec) rec->LAM[iter] = w.lambda;

    // Position correction with s_corr and plane projection (core.cpp:334-398).
#pragma omp parallel for
    for (long long i = 0; i < N; ++i) {
      const T xi = w.px[i], yi = w.py[i], zi = w.pz[i];
      const T li = w.lambda[i];
      T ax = T(0), ay = T(0), az = T(0);
      for (int64_t k = w.nbr_begin[i]; k < w.nbr_begin[i + 1]; ++k) {
        const int j = w.nbr[k];
        const T ddx = xi - w.px[j];
        const T ddy = yi - w.py[j];
        const T ddz = zi - w.pz[j];
        const T r2 = ddx * ddx + ddy * ddy + ddz * ddz;
        if (r2 < h2) {
          const T r = std::sqrt(r2 < c.min_r2 ? c.min_r2 : r2);
          const T gf = spiky_factor<T>(r, h);
          T s = li + w.lambda[j];
          if (c.scorr && c.scorr_inv_wdq > T(0)) {
            const T W = poly6<T>(r2, h);
            const T ratio = W * c.scorr_inv_wdq;
            s += -c.scorr_k * pow_n<T>(ratio, c.scorr_n);
          }
          ax += s * gf * ddx;
          ay += s * gf * ddy;
          az += s * gf * ddz;
        }
      }
      ax *= c.inv_density;
      ay *= c.inv_density;
      az *= c.inv_density;
      if (rec) {
        rec->Q[iter][i] = xi + ax;
        rec->Q[iter][n + i] = yi + ay;
        rec->Q[iter][2 * n + i] = zi + az;
      }
      if (p.plane_count > 0) {
        T qx = xi + ax, qy = yi + ay, qz = zi + az;
        for (int q = 0; q < p.plane_count; ++q) {
          const T nx = T(p.plane_nx[q]), ny = T(p.plane_ny[q]),
                  nz = T(p.plane_nz[q]), d = T(p.plane_d[q]);
          const T sd = nx * qx + ny * qy + nz * qz - d;
          const T pen = -sd;
          if (pen > T(0)) {
            qx += nx * pen;
            qy += ny * pen;
            qz += nz * pen;
          }
        }
        ax = qx - xi;
        ay = qy - yi;
        az = qz - zi;
      }
      w.dx[i] = ax;
      w.dy[i] = ay;
      w.dz[i] = az;
    }
#pragma omp parallel for
    for (long long i = 0; i < N; ++i) {  // core.cpp:400-407
      w.px[i] += w.dx[i];
      w.py[i] += w.dy[i];
      w.pz[i] += w.dz[i];
    }
    if (rec) put3(rec->P[iter + 1], n, w.px.data(), w.py.data(), w.pz.data());
  }
  if (rec) rec->rho = w.rho;

  // Commit (core.cpp:410-421).
#pragma omp parallel for
  for (long long i = 0; i < N; ++i) {
    VX[i] = (w.px[i] - X[i]) / dt;
    VY[i] = (w.py[i] - Y[i]) / dt;
    VZ[i] = (w.pz[i] - Z[i]) / dt;
    X[i] = w.px[i];
    Y[i] = w.py[i];
    Z[i] = w.pz[i];
  }
  if (rec) {
    put3(rec->x1, n, X, Y, Z);
    put3(rec->v2, n, VX, VY, VZ);
  }

  // XSPH viscosity over the step's lists at committed positions (core.cpp:423-466).
  if (p.enable_xsph && p.visc_c != 0.0f) {
    const T cvis = T(p.visc_c);
#pragma omp parallel for
    for (long long i = 0; i < N; ++i) {
      const T vx = VX[i], vy = VY[i], vz = VZ[i];
      T sx = T(0), sy = T(0), sz = T(0);
      for (int64_t k = w.nbr_begin[i]; k < w.nbr_begin[i + 1]; ++k) {
        const int j = w.nbr[k];
        const T ddx = X[i] - X[j];
        const T ddy = Y[i] - Y[j];
        const T ddz = Z[i] - Z[j];
        const T r2 = ddx * ddx + ddy * ddy + ddz * ddz;
        if (r2 < h2) {
          const T W = poly6<T>(r2, h);
          const T inv_rho_j = (w.rho[j] > T(0)) ? (c.mass / w.rho[j]) : T(0);
          sx += (VX[j] - vx) * W * inv_rho_j;
          sy += (VY[j] - vy) * W * inv_rho_j;
          sz += (VZ[j] - vz) * W * inv_rho_j;
        }
      }
      w.dvx[i] = sx;
      w.dvy[i] = sy;
      w.dvz[i] = sz;
    }
#pragma omp parallel for
    for (long long i = 0; i < N; ++i) {
      VX[i] += cvis * w.dvx[i];
      VY[i] += cvis * w.dvy[i];
      VZ[i] += cvis * w.dvz[i];
    }
  }

  if (rec) put3(rec->v3, n, VX, VY, VZ);

  // Vorticity confinement (core.cpp:468-571).
  if (p.enable_vorticity && p.vort_epsilon != 0.0f) {
#pragma omp parallel for
    for (long long i = 0; i < N; ++i) {
      const T xi = X[i], yi = Y[i], zi = Z[i];
      const T vx = VX[i], vy = VY[i], vz = VZ[i];
      T ax = T(0), ay = T(0), az = T(0);
      for (int64_t k = w.nbr_begin[i]; k < w.nbr_begin[i + 1]; ++k) {
        const int j = w.nbr[k];
        const T ddx = xi - X[j];
        const T ddy = yi - Y[j];
        const T ddz = zi - Z[j];
        const T r2 = ddx * ddx + ddy * ddy + ddz * ddz;
        if (r2 < h2) {
          const T r = std::sqrt(r2 < c.min_r2 ? c.min_r2 : r2);
          const T gf = spiky_factor<T>(r, h);
          const T gx = gf * ddx, gy = gf * ddy, gz = gf * ddz;
          const T ux = VX[j] - vx, uy = VY[j] - vy, uz = VZ[j] - vz;
          ax += uy * gz - uz * gy;
          ay += uz * gx - ux * gz;
          az += ux * gy - uy * gx;
        }
      }
      w.ox[i] = ax;
      w.oy[i] = ay;
      w.oz[i] = az;
      w.omag[i] = std::sqrt(ax * ax + ay * ay + az * az);
    }
    if (rec) {
      put3(rec->om, n, w.ox.data(), w.oy.data(), w.oz.data());
      rec->omag = w.omag;
    }
#pragma omp parallel for
    for (long long i = 0; i < N; ++i) {
      const T xi = X[i], yi = Y[i], zi = Z[i];
      const T mi = w.omag[i];
      T ax = T(0), ay = T(0), az = T(0);
      for (int64_t k = w.nbr_begin[i]; k < w.nbr_begin[i + 1]; ++k) {
        const int j = w.nbr[k];
        const T ddx = xi - X[j];
        const T ddy = yi - Y[j];
        const T ddz = zi - Z[j];
        const T r2 = ddx * ddx + ddy * ddy + ddz * ddz;
        if (r2 < h2) {
          const T r = std::sqrt(r2 < c.min_r2 ? c.min_r2 : r2);
          const T gf = spiky_factor<T>(r, h);
          const T coeff = w.omag[j] - mi;
          ax += coeff * (gf * ddx);
          ay += coeff * (gf * ddy);
          az += coeff * (gf * ddz);
        }
      }
      w.ex[i] = ax;
      w.ey[i] = ay;
      w.ez[i] = az;
    }
    const T veps = T(p.vort_epsilon);
    const T neps = T(p.vort_norm_eps);
#pragma omp parallel for
    for (long long i = 0; i < N; ++i) {
      const T ex = w.ex[i], ey = w.ey[i], ez = w.ez[i];
      const T len = std::sqrt(ex * ex + ey * ey + ez * ez);
      T nx = T(0), ny = T(0), nz = T(0);
      if (len > neps) {
        const T inv = T(1) / len;
        nx = ex * inv;
        ny = ey * inv;
        nz = ez * inv;
      }
      const T ox = w.ox[i], oy = w.oy[i], oz = w.oz[i];
      const T fxv = veps * (ny * oz - nz * oy);
      const T fyv = veps * (nz * ox - nx * oz);
      const T fzv = veps * (nx * oy - ny * ox);
      VX[i] += dt * fxv;
      VY[i] += dt * fyv;
      VZ[i] += dt * fzv;
    }
  }

  // Plane restitution and friction (core.cpp:573-612).
  if (contacts_on(p)) {
    const T e = T(p.plane_restitution);
    T scale[FLUID_MAX_PLANES];
    for (int q = 0; q < p.plane_count; ++q) scale[q] = T(1) - T(plane_mu(p, q));
#pragma omp parallel for
    for (long long i = 0; i < N; ++i) {
      T vx = VX[i], vy = VY[i], vz = VZ[i];
      const T xi = X[i], yi = Y[i], zi = Z[i];
      for (int q = 0; q < p.plane_count; ++q) {
        const T nx = T(p.plane_nx[q]), ny = T(p.plane_ny[q]),
                nz = T(p.plane_nz[q]), d = T(p.plane_d[q]);
        const T sd = nx * xi + ny * yi + nz * zi - d;
        if (sd <= T(0)) {
          const T vn = nx * vx + ny * vy + nz * vz;
          T vn_new = vn;
          if (vn < T(0)) vn_new = -e * vn;
          const T tx = vx - vn * nx;
          const T ty = vy - vn * ny;
          const T tz = vz - vn * nz;
          vx = tx * scale[q] + vn_new * nx;
          vy = ty * scale[q] + vn_new * ny;
          vz = tz * scale[q] + vn_new * nz;
        }
      }
      VX[i] = vx;
      VY[i] = vy;
      VZ[i] = vz;
    }
  }

  *time += dt;  // core.cpp:614

  int64_t pairs = static_cast<int64_t>(w.nbr.size());
  int32_t mx = 0;
  for (std::size_t i = 0; i < n; ++i) {
    mx = std::max<int32_t>(mx, static_cast<int32_t>(w.nbr_begin[i + 1] - w.nbr_begin[i]));
  }
  if (pairs_out) *pairs_out = pairs;
  if (max_out) *max_out = mx;
  if (dump) {
    for (std::size_t i = 0; i < n; ++i) {
      if (dump->cell_keys) {
        const Cell k = grid ? w.key[i] : cell_of(w.px[i], w.py[i], w.pz[i], h);
        dump->cell_keys[3 * i + 0] = k.x;
        dump->cell_keys[3 * i + 1] = k.y;
        dump->cell_keys[3 * i + 2] = k.z;
      }
      if (dump->sorted_order) dump->sorted_order[i] = grid ? w.order[i] : int32_t(i);
      if (dump->neighbor_counts)
        dump->neighbor_counts[i] = static_cast<int32_t>(w.nbr_begin[i + 1] - w.nbr_begin[i]);
      if (dump->rho) dump->rho[i] = w.rho[i];
      if (dump->lambda) dump->lambda[i] = w.lambda[i];
    }
  }
  return 0;
}

template <typename A, typename B>
Record<B> convert_record(const Record<A>& r) {
  Record<B> o;
  o.n = r.n;
  o.iters = r.iters;
  o.vorticity = r.vorticity;
  auto cv = [](const std::vector<A>& v) { return std::vector<B>(v.begin(), v.end()); };
  o.x0 = cv(r.x0);
  o.x1 = cv(r.x1);
  o.v2 = cv(r.v2);
  o.rho = cv(r.rho);
  o.v3 = cv(r.v3);
  o.om = cv(r.om);
  o.omag = cv(r.omag);
  for (const auto& v : r.P) o.P.push_back(cv(v));
  for (const auto& v : r.Q) o.Q.push_back(cv(v));
  for (const auto& v : r.LAM) o.LAM.push_back(cv(v));
  o.nbr = r.nbr;
  o.nbr_begin = r.nbr_begin;
  return o;
}

// Reverse-mode derivative of one recorded step. Given the cotangents of the
// step's outputs (positions gxo, velocities gvo; SoA 3n), accumulates those of
// its inputs (gxi, gvi) and of the XSPH coefficient (*gc). Neighbour sets and
// every branch (r < h, the min_r clamp, plane contacts, restitution's
// vn < 0) are held at the recorded forward's values. Membership is symmetric
// (r^2 of (i, j) and (j, i) are the same float), so each transposed sum is a
// gather over i's own list.
template <typename T>
int adjoint(const Record<T>& R, const fluid_params& p, const T* gxo, const T* gvo, T* gxi, T* gvi, T* gc) {
  const std::size_t n = R.n;
  const long long N = static_cast<long long>(n);
  const int K = R.iters;
  const Consts<T> c = make_consts<T>(p);
  const T h = c.h, h2 = c.h2, dt = c.dt, m = c.mass, gs = c.grad_scale, ir = c.inv_density;
  const T pi = Pi<T>::value;
  const T h2_ = h * h, h4 = h2_ * h2_, h9 = h4 * h4 * h;
  const T c6 = T(315) / (T(64) * pi * h9);
  const T csp = T(-45) / (pi * h2_ * h2_ * h2_);
  const T W0 = c6 * h2 * h2 * h2;
  const bool scorr = c.scorr && c.scorr_inv_wdq > T(0);
  const T nk = -c.scorr_k, iw = c.scorr_inv_wdq;
  const int sn = c.scorr_n;
  const bool xsph = p.enable_xsph && p.visc_c != 0.0f;
  const T cv = T(p.visc_c);
  const bool rest = contacts_on(p);
  const T e = T(p.plane_restitution);
  T mu_s[FLUID_MAX_PLANES];
  for (int q = 0; q < p.plane_count; ++q) mu_s[q] = T(1) - T(plane_mu(p, q));
  auto W = [&](T r2) { const T d = h2 - r2; return c6 * d * d * d; };
  auto dW = [&](T r2) { const T d = h2 - r2; return T(-3) * c6 * d * d; };
  auto F = [&](T r) { const T d = h - r; return csp * d * d; };
  auto dF = [&](T r) { return T(-2) * csp * (h - r); };
  auto powr = [&](T x, int k) { T y = T(1); for (int q = 0; q < k; ++q) y *= x; return y; };
  auto at = [n](const std::vector<T>& a, std::size_t i, int d) { return a[d * n + i]; };

  const bool vort = R.vorticity;
  const T ve = T(p.vort_epsilon), vne = T(p.vort_norm_eps);
  std::vector<T> gx1(gxo, gxo + 3 * n), gv3(3 * n), gv2(3 * n), dv(3 * n, T(0)), grho(n, T(0));
  std::vector<T> gv4(3 * n), eb(3 * n, T(0)), obd(3 * n, T(0)), ob(3 * n, T(0));
  std::vector<T> aj(n);
  for (std::size_t i = 0; i < n; ++i) aj[i] = (R.rho[i] > T(0)) ? m / R.rho[i] : T(0);

  // XSPH sums, then restitution reversed (core.cpp:423-466, 573-612).
#pragma omp parallel for
  for (long long ii = 0; ii < N; ++ii) {
    const std::size_t i = static_cast<std::size_t>(ii);
    T s[3] = {0, 0, 0};
    if (xsph) {
      for (int64_t k = R.nbr_begin[i]; k < R.nbr_begin[i + 1]; ++k) {
        const std::size_t j = static_cast<std::size_t>(R.nbr[k]);
        T d[3], r2 = 0;
        for (int a = 0; a < 3; ++a) { d[a] = at(R.x1, i, a) - at(R.x1, j, a); r2 += d[a] * d[a]; }
        if (r2 < h2) {
          const T w = W(r2);
          for (int a = 0; a < 3; ++a) s[a] += (at(R.v2, j, a) - at(R.v2, i, a)) * w * aj[j];
        }
      }
    }
    T v[3], g[3], Nv[3] = {0, 0, 0}, eta[3] = {0, 0, 0}, elen = 0;
    for (int a = 0; a < 3; ++a) {
      dv[a * n + i] = s[a];
      v[a] = at(R.v2, i, a) + cv * s[a];
      g[a] = gvo[a * n + i];
    }
    const T om[3] = {vort ? at(R.om, i, 0) : T(0), vort ? at(R.om, i, 1) : T(0), vort ? at(R.om, i, 2) : T(0)};
    if (vort) {  // eta, N, confinement force (core.cpp:512-570)
      for (int64_t k = R.nbr_begin[i]; k < R.nbr_begin[i + 1]; ++k) {
        const std::size_t j = static_cast<std::size_t>(R.nbr[k]);
        T d[3], r2 = 0;
        for (int a = 0; a < 3; ++a) { d[a] = at(R.x1, i, a) - at(R.x1, j, a); r2 += d[a] * d[a]; }
        if (!(r2 < h2)) continue;
        const T f = F(std::sqrt(r2 < c.min_r2 ? c.min_r2 : r2));
        for (int a = 0; a < 3; ++a) eta[a] += (R.omag[j] - R.omag[i]) * (f * d[a]);
      }
      elen = std::sqrt(eta[0] * eta[0] + eta[1] * eta[1] + eta[2] * eta[2]);
      if (elen > vne)
        for (int a = 0; a < 3; ++a) Nv[a] = eta[a] / elen;
      const T fv[3] = {ve * (Nv[1] * om[2] - Nv[2] * om[1]), ve * (Nv[2] * om[0] - Nv[0] * om[2]),
                       ve * (Nv[0] * om[1] - Nv[1] * om[0])};
      for (int a = 0; a < 3; ++a) v[a] += dt * fv[a];
    }
    if (rest) {
      bool act[FLUID_MAX_PLANES];
      T sc[FLUID_MAX_PLANES];
      for (int q = 0; q < p.plane_count; ++q) {
        const T nq[3] = {T(p.plane_nx[q]), T(p.plane_ny[q]), T(p.plane_nz[q])};
        const T sd = nq[0] * at(R.x1, i, 0) + nq[1] * at(R.x1, i, 1) + nq[2] * at(R.x1, i, 2) - T(p.plane_d[q]);
        act[q] = sd <= T(0);
        if (act[q]) {
          const T vn = nq[0] * v[0] + nq[1] * v[1] + nq[2] * v[2];
          sc[q] = (vn < T(0)) ? -e : T(1);
          for (int a = 0; a < 3; ++a) v[a] = (v[a] - vn * nq[a]) * mu_s[q] + sc[q] * vn * nq[a];
        }
      }
      for (int q = p.plane_count - 1; q >= 0; --q) {
        if (!act[q]) continue;
        const T nq[3] = {T(p.plane_nx[q]), T(p.plane_ny[q]), T(p.plane_nz[q])};
        const T gn = nq[0] * g[0] + nq[1] * g[1] + nq[2] * g[2];
        for (int a = 0; a < 3; ++a) g[a] = mu_s[q] * g[a] + (sc[q] - mu_s[q]) * gn * nq[a];
      }
    }
    for (int a = 0; a < 3; ++a) gv4[a * n + i] = g[a];
    if (vort) {  // f = eps N x omega reversed; N = eta/|eta| reversed
      const T fb[3] = {dt * g[0], dt * g[1], dt * g[2]};
      const T Nb[3] = {ve * (om[1] * fb[2] - om[2] * fb[1]), ve * (om[2] * fb[0] - om[0] * fb[2]),
                       ve * (om[0] * fb[1] - om[1] * fb[0])};
      obd[i] = ve * (fb[1] * Nv[2] - fb[2] * Nv[1]);
      obd[n + i] = ve * (fb[2] * Nv[0] - fb[0] * Nv[2]);
      obd[2 * n + i] = ve * (fb[0] * Nv[1] - fb[1] * Nv[0]);
      if (elen > vne) {
        const T nn = Nv[0] * Nb[0] + Nv[1] * Nb[1] + Nv[2] * Nb[2];
        for (int a = 0; a < 3; ++a) eb[a * n + i] = (Nb[a] - Nv[a] * nn) / elen;
      }
    }
  }
  if (vort) {
    // eta = sum (|w_j| - |w_i|) g_ij reversed: |w| and positions.
#pragma omp parallel for
    for (long long ii = 0; ii < N; ++ii) {
      const std::size_t i = static_cast<std::size_t>(ii);
      T mb = 0, add[3] = {0, 0, 0};
      for (int64_t k = R.nbr_begin[i]; k < R.nbr_begin[i + 1]; ++k) {
        const std::size_t j = static_cast<std::size_t>(R.nbr[k]);
        T d[3], r2 = 0;
        for (int a = 0; a < 3; ++a) { d[a] = at(R.x1, i, a) - at(R.x1, j, a); r2 += d[a] * d[a]; }
        if (!(r2 < h2)) continue;
        const bool clamp = r2 < c.min_r2;
        const T r = std::sqrt(clamp ? c.min_r2 : r2);
        const T f = F(r), fpr = clamp ? T(0) : dF(r) / r;
        T e[3], de = 0;
        for (int a = 0; a < 3; ++a) { e[a] = eb[a * n + i] + eb[a * n + j]; de += d[a] * e[a]; }
        mb -= f * de;
        const T dm = R.omag[j] - R.omag[i];
        for (int a = 0; a < 3; ++a) add[a] += dm * (f * e[a] + fpr * de * d[a]);
      }
      const T m = R.omag[i];
      for (int a = 0; a < 3; ++a) {
        ob[a * n + i] = obd[a * n + i] + (m > T(0) ? mb * at(R.om, i, a) / m : T(0));
        gx1[a * n + i] += add[a];
      }
    }
    // omega = sum (u_j - u_i) x g_ij reversed: velocities after XSPH and positions.
#pragma omp parallel for
    for (long long ii = 0; ii < N; ++ii) {
      const std::size_t i = static_cast<std::size_t>(ii);
      T gu[3] = {gv4[i], gv4[n + i], gv4[2 * n + i]}, add[3] = {0, 0, 0};
      for (int64_t k = R.nbr_begin[i]; k < R.nbr_begin[i + 1]; ++k) {
        const std::size_t j = static_cast<std::size_t>(R.nbr[k]);
        T d[3], r2 = 0;
        for (int a = 0; a < 3; ++a) { d[a] = at(R.x1, i, a) - at(R.x1, j, a); r2 += d[a] * d[a]; }
        if (!(r2 < h2)) continue;
        const bool clamp = r2 < c.min_r2;
        const T r = std::sqrt(clamp ? c.min_r2 : r2);
        const T f = F(r), fpr = clamp ? T(0) : dF(r) / r;
        const T o[3] = {ob[i] + ob[j], ob[n + i] + ob[n + j], ob[2 * n + i] + ob[2 * n + j]};
        const T g[3] = {f * d[0], f * d[1], f * d[2]};
        gu[0] -= g[1] * o[2] - g[2] * o[1];
        gu[1] -= g[2] * o[0] - g[0] * o[2];
        gu[2] -= g[0] * o[1] - g[1] * o[0];
        const T w[3] = {at(R.v3, j, 0) - at(R.v3, i, 0), at(R.v3, j, 1) - at(R.v3, i, 1),
                        at(R.v3, j, 2) - at(R.v3, i, 2)};
        const T C[3] = {o[1] * w[2] - o[2] * w[1], o[2] * w[0] - o[0] * w[2], o[0] * w[1] - o[1] * w[0]};
        const T cd = C[0] * d[0] + C[1] * d[1] + C[2] * d[2];
        for (int a = 0; a < 3; ++a) add[a] += f * C[a] + fpr * cd * d[a];
      }
      for (int a = 0; a < 3; ++a) {
        gv3[a * n + i] = gu[a];
        gx1[a * n + i] += add[a];
      }
    }
  } else {
    gv3 = gv4;
  }
  if (xsph) {
    T acc = 0;
    for (std::size_t i = 0; i < 3 * n; ++i) acc += gv3[i] * dv[i];
    *gc += cv == T(0) ? T(0) : acc;
  }

  // XSPH reversed.
#pragma omp parallel for
  for (long long ii = 0; ii < N; ++ii) {
    const std::size_t i = static_cast<std::size_t>(ii);
    T g2[3], gx[3] = {0, 0, 0}, rsum = 0;
    for (int a = 0; a < 3; ++a) g2[a] = gv3[a * n + i];
    if (xsph) {
      T wsum = 0, vsum[3] = {0, 0, 0};
      for (int64_t k = R.nbr_begin[i]; k < R.nbr_begin[i + 1]; ++k) {
        const std::size_t j = static_cast<std::size_t>(R.nbr[k]);
        T d[3], r2 = 0;
        for (int a = 0; a < 3; ++a) { d[a] = at(R.x1, i, a) - at(R.x1, j, a); r2 += d[a] * d[a]; }
        if (!(r2 < h2)) continue;
        const T w = W(r2), w1 = dW(r2);
        T ti = 0, tj = 0, tr = 0;
        for (int a = 0; a < 3; ++a) {
          const T dvij = at(R.v2, j, a) - at(R.v2, i, a);
          ti += dvij * gv3[a * n + i];
          tj += -dvij * gv3[a * n + j];
          tr += -dvij * gv3[a * n + j];
        }
        wsum += w * aj[j];
        for (int a = 0; a < 3; ++a) vsum[a] += w * gv3[a * n + j];
        const T coef = T(2) * w1 * cv * (aj[j] * ti + aj[i] * tj);
        for (int a = 0; a < 3; ++a) gx[a] += coef * d[a];
        rsum += w * tr;
      }
      for (int a = 0; a < 3; ++a) g2[a] = gv3[a * n + i] - cv * wsum * gv3[a * n + i] + cv * aj[i] * vsum[a];
      grho[i] = (R.rho[i] > T(0)) ? -(m / (R.rho[i] * R.rho[i])) * cv * rsum : T(0);
    }
    for (int a = 0; a < 3; ++a) {
      gv2[a * n + i] = g2[a];
      gx1[a * n + i] += gx[a];
    }
  }

  // Commit reversed: v2 = (p^K - x0)/dt, x1 = p^K.
  std::vector<T> gP(3 * n), gx0(3 * n), gD(3 * n), gL(n), G(3 * n), gS(n), gRT(n);
  for (std::size_t i = 0; i < 3 * n; ++i) {
    gP[i] = gx1[i] + gv2[i] / dt;
    gx0[i] = -gv2[i] / dt;
  }

  for (int it = K - 1; it >= 0; --it) {
    const auto& P = R.P[it];
    const auto& Q = R.Q[it];
    const auto& L = R.LAM[it];
    // Plane projection reversed (core.cpp:372-393): q -> q + n max(0, -(n.q - d)).
#pragma omp parallel for
    for (long long ii = 0; ii < N; ++ii) {
      const std::size_t i = static_cast<std::size_t>(ii);
      T q[3] = {at(Q, i, 0), at(Q, i, 1), at(Q, i, 2)}, g[3];
      for (int a = 0; a < 3; ++a) g[a] = gP[a * n + i];
      bool act[FLUID_MAX_PLANES];
      for (int k = 0; k < p.plane_count; ++k) {
        const T nq[3] = {T(p.plane_nx[k]), T(p.plane_ny[k]), T(p.plane_nz[k])};
        const T pen = -(nq[0] * q[0] + nq[1] * q[1] + nq[2] * q[2] - T(p.plane_d[k]));
        act[k] = pen > T(0);
        if (act[k]) for (int a = 0; a < 3; ++a) q[a] += nq[a] * pen;
      }
      for (int k = p.plane_count - 1; k >= 0; --k) {
        if (!act[k]) continue;
        const T nq[3] = {T(p.plane_nx[k]), T(p.plane_ny[k]), T(p.plane_nz[k])};
        const T gn = nq[0] * g[0] + nq[1] * g[1] + nq[2] * g[2];
        for (int a = 0; a < 3; ++a) g[a] -= gn * nq[a];
      }
      for (int a = 0; a < 3; ++a) gD[a * n + i] = g[a];
    }
    // Position correction reversed (core.cpp:334-370) and lambda recomputed.
#pragma omp parallel for
    for (long long ii = 0; ii < N; ++ii) {
      const std::size_t i = static_cast<std::size_t>(ii);
      T gp[3], gl = 0, rs = 0, Gi[3] = {0, 0, 0}, s1 = 0;
      for (int a = 0; a < 3; ++a) gp[a] = gD[a * n + i];
      for (int64_t k = R.nbr_begin[i]; k < R.nbr_begin[i + 1]; ++k) {
        const std::size_t j = static_cast<std::size_t>(R.nbr[k]);
        T d[3], r2 = 0;
        for (int a = 0; a < 3; ++a) { d[a] = at(P, i, a) - at(P, j, a); r2 += d[a] * d[a]; }
        if (!(r2 < h2)) continue;
        const bool clamp = r2 < c.min_r2;
        const T r = std::sqrt(clamp ? c.min_r2 : r2);
        const T f = F(r), fpr = clamp ? T(0) : dF(r) / r;
        T s = L[i] + L[j], alpha = s * fpr;
        if (scorr) {
          const T x = W(r2) * iw;
          s += nk * powr(x, sn);
          alpha = s * fpr + T(2) * f * nk * T(sn) * powr(x, sn - 1) * iw * dW(r2);
        }
        T de = 0;
        for (int a = 0; a < 3; ++a) de += d[a] * (gD[a * n + i] - gD[a * n + j]);
        for (int a = 0; a < 3; ++a) gp[a] += ir * (s * f * (gD[a * n + i] - gD[a * n + j]) + alpha * de * d[a]);
        gl += ir * f * de;
        rs += W(r2);
        for (int a = 0; a < 3; ++a) Gi[a] += f * d[a];
        s1 += f * f * r2;
      }
      const T rho = m * (rs + W0);
      const T C = rho * ir - T(1);
      const T S = gs * gs * (s1 + Gi[0] * Gi[0] + Gi[1] * Gi[1] + Gi[2] * Gi[2]);
      const T lam = -C / (S + c.epsilon);
      const T gC = -gl / (S + c.epsilon);
      gS[i] = -gl * lam / (S + c.epsilon);
      gRT[i] = (it == K - 1 ? grho[i] : T(0)) + gC * ir;
      for (int a = 0; a < 3; ++a) {
        G[a * n + i] = Gi[a];
        gP[a * n + i] = gp[a];  // partial: direct + correction terms; lambda terms next
      }
      gL[i] = gl;
    }
    // Lambda reversed (core.cpp:281-329), gathered over i's list.
#pragma omp parallel for
    for (long long ii = 0; ii < N; ++ii) {
      const std::size_t i = static_cast<std::size_t>(ii);
      T add[3] = {0, 0, 0};
      for (int64_t k = R.nbr_begin[i]; k < R.nbr_begin[i + 1]; ++k) {
        const std::size_t j = static_cast<std::size_t>(R.nbr[k]);
        T d[3], r2 = 0;
        for (int a = 0; a < 3; ++a) { d[a] = at(P, i, a) - at(P, j, a); r2 += d[a] * d[a]; }
        if (!(r2 < h2)) continue;
        const bool clamp = r2 < c.min_r2;
        const T r = std::sqrt(clamp ? c.min_r2 : r2);
        const T f = F(r), fpr = clamp ? T(0) : dF(r) / r;
        T dGi = 0, dGj = 0;
        for (int a = 0; a < 3; ++a) { dGi += d[a] * G[a * n + i]; dGj += d[a] * G[a * n + j]; }
        const T t1 = T(2) * m * dW(r2) * (gRT[i] + gRT[j]);
        const T t2 = gs * gs * (gS[i] + gS[j]) * (T(2) * f * fpr * r2 + T(2) * f * f);
        const T t4 = T(2) * gs * gs * fpr * (gS[i] * dGi - gS[j] * dGj);
        for (int a = 0; a < 3; ++a)
          add[a] += (t1 + t2 + t4) * d[a] + T(2) * f * gs * gs * (gS[i] * G[a * n + i] - gS[j] * G[a * n + j]);
      }
      for (int a = 0; a < 3; ++a) gP[a * n + i] += add[a];
    }
  }

  // Predict reversed: p^0 = x0 + (v + f dt) dt.
  for (std::size_t i = 0; i < 3 * n; ++i) {
    gxi[i] += gx0[i] + gP[i];
    gvi[i] += gP[i] * dt;
  }
  return FLUID_OK;
}

bool params_ok(const fluid_params* p) {
  return p && p->plane_count >= 0 && p->plane_count <= FLUID_MAX_PLANES &&
         p->solver_iterations >= 0;
}

}  // namespace

extern "C" {

typedef struct pbf_oracle_dump_f32 {
  int32_t* cell_keys;       // 3 per particle, cells of p* (core.cpp:165-171)
  int32_t* sorted_order;    // particle at each sorted position (core.cpp:173-183)
  int32_t* neighbor_counts; // per particle (core.cpp:245-246)
  float* rho;               // last lambda pass (core.cpp:321)
  float* lambda;            // last lambda pass (core.cpp:328)
} pbf_oracle_dump_f32;

typedef struct pbf_oracle_dump_f64 {
  int32_t* cell_keys;
  int32_t* sorted_order;
  int32_t* neighbor_counts;
  double* rho;
  double* lambda;
} pbf_oracle_dump_f64;

void* pbf_oracle_create_f32(void) { return new Workspace<float>(); }
void pbf_oracle_destroy_f32(void* ws) { delete static_cast<Workspace<float>*>(ws); }
void* pbf_oracle_create_f64(void) { return new Workspace<double>(); }
void pbf_oracle_destroy_f64(void* ws) { delete static_cast<Workspace<double>*>(ws); }

int pbf_oracle_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
  return omp_get_max_threads();
#else
  (void)n;
  return 1;
#endif
}

// Runs `nsteps` steps. Optional per-step records (length nsteps, may be NULL):
// neighbour pairs, largest neighbour count, and mean / max of rho_i/rho0 - 1
// from the last lambda pass. The dump (may be NULL) describes the last step.
int pbf_oracle_run_f32(void* ws, const fluid_params* p, int64_t count,
                       float* px, float* py, float* pz, float* vx, float* vy,
                       float* vz, float* time, int32_t nsteps,
                       const pbf_oracle_dump_f32* dump, int64_t* pairs,
                       int32_t* nmax, double* dens_mean, double* dens_max) {
  if (!ws || !params_ok(p) || count < 0 || nsteps < 0) return FLUID_ERR_INVALID_ARGUMENT;
  auto& w = *static_cast<Workspace<float>*>(ws);
  const std::size_t n = static_cast<std::size_t>(count);
  for (int s = 0; s < nsteps; ++s) {
    Dump<float> d{};
    if (dump) d = Dump<float>{dump->cell_keys, dump->sorted_order, dump->neighbor_counts, dump->rho, dump->lambda};
    step<float>(w, *p, n, px, py, pz, vx, vy, vz, time, (dump && s == nsteps - 1) ? &d : nullptr,
                pairs ? &pairs[s] : nullptr, nmax ? &nmax[s] : nullptr);
    if (dens_mean || dens_max) {
      double sum = 0.0, mx = -1e300;
      for (std::size_t i = 0; i < n; ++i) {
        const double e = double(w.rho[i]) / double(p->density) - 1.0;
        sum += e;
        mx = std::max(mx, e);
      }
      if (dens_mean) dens_mean[s] = n ? sum / double(n) : 0.0;
      if (dens_max) dens_max[s] = n ? mx : 0.0;
    }
  }
  return FLUID_OK;
}

int pbf_oracle_run_f64(void* ws, const fluid_params* p, int64_t count,
                       double* px, double* py, double* pz, double* vx,
                       double* vy, double* vz, double* time, int32_t nsteps,
                       const pbf_oracle_dump_f64* dump, int64_t* pairs,
                       int32_t* nmax, double* dens_mean, double* dens_max) {
  if (!ws || !params_ok(p) || count < 0 || nsteps < 0) return FLUID_ERR_INVALID_ARGUMENT;
  auto& w = *static_cast<Workspace<double>*>(ws);
  const std::size_t n = static_cast<std::size_t>(count);
  for (int s = 0; s < nsteps; ++s) {
    Dump<double> d{};
    if (dump) d = Dump<double>{dump->cell_keys, dump->sorted_order, dump->neighbor_counts, dump->rho, dump->lambda};
    step<double>(w, *p, n, px, py, pz, vx, vy, vz, time, (dump && s == nsteps - 1) ? &d : nullptr,
                 pairs ? &pairs[s] : nullptr, nmax ? &nmax[s] : nullptr);
    if (dens_mean || dens_max) {
      double sum = 0.0, mx = -1e300;
      for (std::size_t i = 0; i < n; ++i) {
        const double e = w.rho[i] / double(p->density) - 1.0;
        sum += e;
        mx = std::max(mx, e);
      }
      if (dens_mean) dens_mean[s] = n ? sum / double(n) : 0.0;
      if (dens_max) dens_max[s] = n ? mx : 0.0;
    }
  }
  return FLUID_OK;
}

// One step's vector-Jacobian product. Runs the forward step from (x, v)
// (SoA 3n each) in float (fwd32 != 0, the trajectory the GPU computes) or
// double, writes its outputs to (x_out, v_out) (same type as the forward),
// then back-propagates the cotangents (gx_out, gv_out) in double arithmetic,
// adding into gx_in, gv_in and *gc (XSPH coefficient).
int pbf_oracle_vjp(const fluid_params* p, int64_t count, int32_t fwd32, const void* x, const void* v,
                   void* x_out, void* v_out, const double* gx_out, const double* gv_out, double* gx_in,
                   double* gv_in, double* gc) {
  if (!params_ok(p) || count < 0) return FLUID_ERR_INVALID_ARGUMENT;
  const std::size_t n = static_cast<std::size_t>(count);
  Record<double> rd;
  if (fwd32) {
    Workspace<float> w;
    std::vector<float> s(6 * n);
    std::copy(static_cast<const float*>(x), static_cast<const float*>(x) + 3 * n, s.begin());
    std::copy(static_cast<const float*>(v), static_cast<const float*>(v) + 3 * n, s.begin() + 3 * n);
    float t = 0.0f;
    Record<float> rf;
    step<float>(w, *p, n, s.data(), s.data() + n, s.data() + 2 * n, s.data() + 3 * n, s.data() + 4 * n,
                s.data() + 5 * n, &t, nullptr, nullptr, nullptr, &rf);
    if (x_out) std::copy(s.begin(), s.begin() + 3 * n, static_cast<float*>(x_out));
    if (v_out) std::copy(s.begin() + 3 * n, s.end(), static_cast<float*>(v_out));
    rd = convert_record<float, double>(rf);
  } else {
    Workspace<double> w;
    std::vector<double> s(6 * n);
    std::copy(static_cast<const double*>(x), static_cast<const double*>(x) + 3 * n, s.begin());
    std::copy(static_cast<const double*>(v), static_cast<const double*>(v) + 3 * n, s.begin() + 3 * n);
    double t = 0.0;
    step<double>(w, *p, n, s.data(), s.data() + n, s.data() + 2 * n, s.data() + 3 * n, s.data() + 4 * n,
                 s.data() + 5 * n, &t, nullptr, nullptr, nullptr, &rd);
    if (x_out) std::copy(s.begin(), s.begin() + 3 * n, static_cast<double*>(x_out));
    if (v_out) std::copy(s.begin() + 3 * n, s.end(), static_cast<double*>(v_out));
  }
  if (n == 0) return FLUID_OK;
  return adjoint<double>(rd, *p, gx_out, gv_out, gx_in, gv_in, gc);
}

}  // extern "C"
