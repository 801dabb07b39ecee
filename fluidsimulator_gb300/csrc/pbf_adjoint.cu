// Adjoint (reverse-mode derivative) of the GB300 PBF timestep.
//
// Runs on the internals a recording forward kept (StepRecord) and the step's
// neighbour lists, which stay valid until the next step. Neighbour sets and
// every branch (r < h, the 0.01 h clamp, plane contacts, restitution's
// vn < 0) are held at the forward's values. Membership is symmetric -- the
// r^2 of (i, j) and (j, i) are the same float -- so each transposed sum
// ("how much does i's output depend on my input") is a gather over the
// particle's own list: no atomics, deterministic results.
//
// Launch order (slot order of the step's output):
//   k_adj_prepare  committed velocity v2 = (p^K - x0)/dt, output cotangents
//                  gathered from caller order
//   k_adj_out      XSPH sum and vorticity force recomputed, restitution
//                  reversed (core.cpp:573-612), confinement force reversed
//   k_adj_eta      eta reversed (core.cpp:512-543)      } vorticity
//   k_adj_omega    omega reversed (core.cpp:472-508)    } confinement
//   k_adj_xsph     XSPH reversed (core.cpp:423-466), commit reversed
//   per iteration k = K-1 .. 0:
//     k_adj_proj    plane projection reversed (core.cpp:372-393)
//     k_adj_delta   position correction reversed (core.cpp:334-370) and the
//                   iteration's density constraint recomputed
//     k_adj_lambda  density constraint reversed (core.cpp:281-329)
//   k_adj_in       prediction reversed (core.cpp:150-161), scattered to
//                  caller order

#include "pbf_adjoint.h"

namespace fgb {
namespace {

constexpr int kAdjBlock = 256;

__device__ __forceinline__ bool adj_failed(const DevStatus* st) {
  return *reinterpret_cast<const volatile int*>(&st->err) != 0;
}

// (x*x + y*y) + z*z with every operation rounded on its own, as the forward's
// membership test computes it, so the adjoint visits exactly the forward's
// pairs (this file is compiled with contraction on).
__device__ __forceinline__ float d2(float x, float y, float z) {
  return __fadd_rn(__fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y)), __fmul_rn(z, z));
}

// Signed distance ((nx x + ny y) + nz z) - d and the projection q += n pen,
// each operation rounded on its own as in the forward (core.cpp:372-393,
// 586-606): contacts decided from recorded positions come out as the
// forward's, also for particles resting exactly on a plane.
__device__ __forceinline__ float plane_sd(const float4 pl, float x, float y, float z) {
  return __fsub_rn(__fadd_rn(__fadd_rn(__fmul_rn(pl.x, x), __fmul_rn(pl.y, y)), __fmul_rn(pl.z, z)), pl.w);
}

// Rows ahead at which a walk over a long recorded list asks the L2 for the
// list (one prefetch per row, on the lane's own entry; nothing for lists
// shorter than that), as the forward's list walkers do.
constexpr int kListAhead = 32;

__device__ __forceinline__ void prefetch_row(const int* p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }

// The recorded lists are 32-bit rows (the forward keeps them so on a step it
// records for the adjoint).
template <typename Body>
__device__ __forceinline__ void for_list(const StepArgs& s, int i, Body&& body) {
  const int n = s.cnt[i];
  const int* __restrict__ list = s.nbr + s.wbase[i >> 5] + (i & 31);
  int k = 0;
  for (; k + 4 <= n; k += 4) {
    if (k + kListAhead + 4 <= n) {
#pragma unroll
      for (int u = 0; u < 4; ++u) prefetch_row(list + 32ll * (k + kListAhead + u));
    }
    const int j0 = __ldcs(list + 32ll * k), j1 = __ldcs(list + 32ll * (k + 1));
    const int j2 = __ldcs(list + 32ll * (k + 2)), j3 = __ldcs(list + 32ll * (k + 3));
    body(j0);
    body(j1);
    body(j2);
    body(j3);
  }
  for (; k < n; ++k) body(__ldcs(list + 32ll * k));
}

// for_list with the neighbours' records fetched four ahead and the next four
// list indices fetched while those are used; body(rec) sees list order.
template <typename Load, typename Body>
__device__ __forceinline__ void for_list_rec(const StepArgs& s, int i, Load&& load, Body&& body) {
  constexpr int kAhead = 4;
  using Rec = decltype(load(0));
  const int n = s.cnt[i];
  const int* __restrict__ list = s.nbr + s.wbase[i >> 5] + (i & 31);
  int k = 0;
  int j[kAhead];
  if (kAhead <= n) {
#pragma unroll
    for (int u = 0; u < kAhead; ++u) j[u] = __ldcs(list + 32ll * u);
  }
  for (; k + kAhead <= n; k += kAhead) {
    Rec r[kAhead];
#pragma unroll
    for (int u = 0; u < kAhead; ++u) r[u] = load(j[u]);
    if (k + 2 * kAhead <= n) {
#pragma unroll
      for (int u = 0; u < kAhead; ++u) j[u] = __ldcs(list + 32ll * (k + kAhead + u));
    }
    if (k + kListAhead + kAhead <= n) {
#pragma unroll
      for (int u = 0; u < kAhead; ++u) prefetch_row(list + 32ll * (k + kListAhead + u));
    }
#pragma unroll
    for (int u = 0; u < kAhead; ++u) body(r[u]);
  }
  for (; k < n; ++k) body(load(__ldcs(list + 32ll * k)));
}

struct Rec2 {
  float4 a, b;
};
struct Rec3 {
  float4 a, b, c;
};

__device__ __forceinline__ float dW(const SceneConst& c, float r2) {  // dW_poly6 / d(r^2)
  const float d = c.h2 - r2;
  return -3.0f * c.poly6_c * d * d;
}
__device__ __forceinline__ float Wp(const SceneConst& c, float r2) {
  const float d = c.h2 - r2;
  return c.poly6_c * d * d * d;
}
__device__ __forceinline__ float Fs(const SceneConst& c, float r) {  // spiky factor
  const float d = c.h - r;
  return c.spiky_c * d * d;
}
__device__ __forceinline__ float dFs(const SceneConst& c, float r) { return -2.0f * c.spiky_c * (c.h - r); }
__device__ __forceinline__ float powi(float x, int k) {
  if (k <= 0) return 1.0f;
  if (k <= 8) {
    float y = x;
    for (int q = 1; q < k; ++q) y *= x;
    return y;
  }
  return powf(x, static_cast<float>(k));
}

__global__ void __launch_bounds__(kAdjBlock) k_adj_prepare(AdjArgs a) {
  if (adj_failed(a.s.status)) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = a.s.n;
  if (i >= n) return;
  const float4 x0 = a.rec.x0[i];
  const float4 pk = a.rec.p[static_cast<size_t>(a.iters) * n + i];
  const float4 p0 = a.rec.p[i];
  const SceneConst& c = a.s.sc[__float_as_int(p0.w)];
  // w: m / rho_i, the XSPH weight of i as a neighbour (core.cpp:446-447).
  const float ri = a.rec.rho[i];
  a.v2[i] = make_float4((pk.x - x0.x) / c.dt, (pk.y - x0.y) / c.dt, (pk.z - x0.z) / c.dt,
                        ri > 0.0f ? c.mass / ri : 0.0f);
  const int o = __float_as_int(x0.w);
  a.gx[i] = make_float4(a.g_pos_out[o], a.g_pos_out[n + o], a.g_pos_out[2 * n + o], 0.0f);
  a.gv[i] = make_float4(a.g_vel_out[o], a.g_vel_out[n + o], a.g_vel_out[2 * n + o], 0.0f);
}

__global__ void __launch_bounds__(kAdjBlock) k_adj_out(AdjArgs a) {
  if (adj_failed(a.s.status)) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = a.s.n;
  if (i >= n) return;
  const float4* __restrict__ x1 = a.rec.p + static_cast<size_t>(a.iters) * n;
  const float4 xi = x1[i];
  const float4 vi = a.v2[i];
  const SceneConst& c = a.s.sc[__float_as_int(a.rec.p[i].w)];
  float sx = 0.0f, sy = 0.0f, sz = 0.0f;
  if (c.xsph_on) {
    auto load = [&](int j) { return Rec2{__ldg(x1 + j), __ldg(a.v2 + j)}; };
    for_list_rec(a.s, i, load, [&](const Rec2 rj) {
      const float4 xj = rj.a;
      const float r2 = d2(xi.x - xj.x, xi.y - xj.y, xi.z - xj.z);
      if (r2 < c.h2) {
        const float4 vj = rj.b;
        const float aj = vj.w;
        const float w = Wp(c, r2) * aj;
        sx += (vj.x - vi.x) * w;
        sy += (vj.y - vi.y) * w;
        sz += (vj.z - vi.z) * w;
      }
    });
  }
  float v[3] = {vi.x + c.visc_c * sx, vi.y + c.visc_c * sy, vi.z + c.visc_c * sz};
  a.dv[i] = make_float4(sx, sy, sz, 0.0f);
  a.v3[i] = make_float4(v[0], v[1], v[2], 0.0f);
  // Vorticity confinement recomputed (core.cpp:512-570): eta from the
  // recorded |omega|, N = eta/|eta|, f = eps N x omega.
  float N[3] = {0.0f, 0.0f, 0.0f}, om[3] = {0.0f, 0.0f, 0.0f}, elen = 0.0f;
  const bool vort = a.vorticity && c.vort_on;
  if (vort) {
    const float4 oi = a.rec.omega[i];
    om[0] = oi.x;
    om[1] = oi.y;
    om[2] = oi.z;
    float ex = 0.0f, ey = 0.0f, ez = 0.0f;
    for_list(a.s, i, [&](int j) {
      const float4 xj = __ldg(x1 + j);
      const float dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
      const float r2 = d2(dx, dy, dz);
      if (!(r2 < c.h2)) return;
      const float f = Fs(c, sqrtf(r2 < c.min_r2 ? c.min_r2 : r2));
      const float dm = __ldg(&a.rec.omega[j].w) - oi.w;
      ex += dm * (f * dx);
      ey += dm * (f * dy);
      ez += dm * (f * dz);
    });
    elen = sqrtf(ex * ex + ey * ey + ez * ez);
    if (elen > c.vort_norm_eps) {
      N[0] = ex / elen;
      N[1] = ey / elen;
      N[2] = ez / elen;
    }
    v[0] += c.dt * (c.vort_eps * (N[1] * om[2] - N[2] * om[1]));
    v[1] += c.dt * (c.vort_eps * (N[2] * om[0] - N[0] * om[2]));
    v[2] += c.dt * (c.vort_eps * (N[0] * om[1] - N[1] * om[0]));
  }
  const float4 go = a.gv[i];
  float g[3] = {go.x, go.y, go.z};
  if (c.rest_on) {
    unsigned act = 0, neg = 0;
    for (int q = 0; q < c.plane_count; ++q) {
      const float4 pl = c.planes[q];
      if (plane_sd(pl, xi.x, xi.y, xi.z) <= 0.0f) {
        act |= 1u << q;
        const float vn = pl.x * v[0] + pl.y * v[1] + pl.z * v[2];
        const float s = vn < 0.0f ? c.rest_neg_e : 1.0f;
        if (vn < 0.0f) neg |= 1u << q;
        const float keep = c.rest_scale[q];
        v[0] = (v[0] - vn * pl.x) * keep + s * vn * pl.x;
        v[1] = (v[1] - vn * pl.y) * keep + s * vn * pl.y;
        v[2] = (v[2] - vn * pl.z) * keep + s * vn * pl.z;
      }
    }
    for (int q = c.plane_count - 1; q >= 0; --q) {
      if (!(act >> q & 1u)) continue;
      const float4 pl = c.planes[q];
      const float s = (neg >> q & 1u) ? c.rest_neg_e : 1.0f;
      const float gn = pl.x * g[0] + pl.y * g[1] + pl.z * g[2];
      const float keep = c.rest_scale[q];
      const float k = (s - keep) * gn;
      g[0] = keep * g[0] + k * pl.x;
      g[1] = keep * g[1] + k * pl.y;
      g[2] = keep * g[2] + k * pl.z;
    }
  }
  if (!a.vorticity) {
    a.gv3[i] = make_float4(g[0], g[1], g[2], 0.0f);
    a.cc[i] = c.xsph_on ? g[0] * sx + g[1] * sy + g[2] * sz : 0.0f;
    return;
  }
  a.gv4[i] = make_float4(g[0], g[1], g[2], 0.0f);
  float ebx = 0.0f, eby = 0.0f, ebz = 0.0f, obx = 0.0f, oby = 0.0f, obz = 0.0f;
  if (vort) {  // f = eps N x omega and N = eta/|eta| reversed
    const float fb[3] = {c.dt * g[0], c.dt * g[1], c.dt * g[2]};
    const float Nb[3] = {c.vort_eps * (om[1] * fb[2] - om[2] * fb[1]), c.vort_eps * (om[2] * fb[0] - om[0] * fb[2]),
                         c.vort_eps * (om[0] * fb[1] - om[1] * fb[0])};
    obx = c.vort_eps * (fb[1] * N[2] - fb[2] * N[1]);
    oby = c.vort_eps * (fb[2] * N[0] - fb[0] * N[2]);
    obz = c.vort_eps * (fb[0] * N[1] - fb[1] * N[0]);
    if (elen > c.vort_norm_eps) {
      const float nn = N[0] * Nb[0] + N[1] * Nb[1] + N[2] * Nb[2];
      ebx = (Nb[0] - N[0] * nn) / elen;
      eby = (Nb[1] - N[1] * nn) / elen;
      ebz = (Nb[2] - N[2] * nn) / elen;
    }
  }
  a.eb[i] = make_float4(ebx, eby, ebz, 0.0f);
  a.obd[i] = make_float4(obx, oby, obz, 0.0f);
}

// eta_i = sum_j (|w_j| - |w_i|) g_ij reversed: cotangent of |omega| and of
// positions; omega's total cotangent.
__global__ void __launch_bounds__(kAdjBlock) k_adj_eta(AdjArgs a) {
  if (adj_failed(a.s.status)) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = a.s.n;
  if (i >= n) return;
  const float4* __restrict__ x1 = a.rec.p + static_cast<size_t>(a.iters) * n;
  const float4 xi = x1[i];
  const SceneConst& c = a.s.sc[__float_as_int(a.rec.p[i].w)];
  const float4 ebi = a.eb[i];
  const float4 oi = c.vort_on ? a.rec.omega[i] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  float mb = 0.0f, ax = 0.0f, ay = 0.0f, az = 0.0f;
  if (c.vort_on) {
    for_list(a.s, i, [&](int j) {
      const float4 xj = __ldg(x1 + j);
      const float dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
      const float r2 = d2(dx, dy, dz);
      if (!(r2 < c.h2)) return;
      const bool clamp = r2 < c.min_r2;
      const float r = sqrtf(clamp ? c.min_r2 : r2);
      const float f = Fs(c, r), fpr = clamp ? 0.0f : dFs(c, r) / r;
      const float4 ebj = __ldg(a.eb + j);
      const float ex = ebi.x + ebj.x, ey = ebi.y + ebj.y, ez = ebi.z + ebj.z;
      const float de = dx * ex + dy * ey + dz * ez;
      mb -= f * de;
      const float dm = __ldg(&a.rec.omega[j].w) - oi.w;
      ax += dm * (f * ex + fpr * de * dx);
      ay += dm * (f * ey + fpr * de * dy);
      az += dm * (f * ez + fpr * de * dz);
    });
  }
  const float4 od = a.obd[i];
  const float k = oi.w > 0.0f ? mb / oi.w : 0.0f;
  a.ob[i] = make_float4(od.x + k * oi.x, od.y + k * oi.y, od.z + k * oi.z, 0.0f);
  float4 gx = a.gx[i];
  gx.x += ax;
  gx.y += ay;
  gx.z += az;
  a.gx[i] = gx;
}

// omega_i = sum_j (u_j - u_i) x g_ij reversed: cotangent of the velocity
// after XSPH and of positions; then dL/dc's per-particle share.
__global__ void __launch_bounds__(kAdjBlock) k_adj_omega(AdjArgs a) {
  if (adj_failed(a.s.status)) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = a.s.n;
  if (i >= n) return;
  const float4* __restrict__ x1 = a.rec.p + static_cast<size_t>(a.iters) * n;
  const float4 xi = x1[i];
  const float4 ui = a.v3[i];
  const SceneConst& c = a.s.sc[__float_as_int(ui.w)];
  const float4 obi = a.ob[i];
  const float4 g4 = a.gv4[i];
  float gu[3] = {g4.x, g4.y, g4.z}, ax = 0.0f, ay = 0.0f, az = 0.0f;
  if (c.vort_on) {
    for_list(a.s, i, [&](int j) {
      const float4 xj = __ldg(x1 + j);
      const float dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
      const float r2 = d2(dx, dy, dz);
      if (!(r2 < c.h2)) return;
      const bool clamp = r2 < c.min_r2;
      const float r = sqrtf(clamp ? c.min_r2 : r2);
      const float f = Fs(c, r), fpr = clamp ? 0.0f : dFs(c, r) / r;
      const float4 obj = __ldg(a.ob + j);
      const float4 uj = __ldg(a.v3 + j);
      const float o[3] = {obi.x + obj.x, obi.y + obj.y, obi.z + obj.z};
      const float g[3] = {f * dx, f * dy, f * dz};
      gu[0] -= g[1] * o[2] - g[2] * o[1];
      gu[1] -= g[2] * o[0] - g[0] * o[2];
      gu[2] -= g[0] * o[1] - g[1] * o[0];
      const float w[3] = {uj.x - ui.x, uj.y - ui.y, uj.z - ui.z};
      const float C[3] = {o[1] * w[2] - o[2] * w[1], o[2] * w[0] - o[0] * w[2], o[0] * w[1] - o[1] * w[0]};
      const float cd = C[0] * dx + C[1] * dy + C[2] * dz;
      ax += f * C[0] + fpr * cd * dx;
      ay += f * C[1] + fpr * cd * dy;
      az += f * C[2] + fpr * cd * dz;
    });
  }
  a.gv3[i] = make_float4(gu[0], gu[1], gu[2], 0.0f);
  const float4 s = a.dv[i];
  a.cc[i] = c.xsph_on ? gu[0] * s.x + gu[1] * s.y + gu[2] * s.z : 0.0f;
  float4 gx = a.gx[i];
  gx.x += ax;
  gx.y += ay;
  gx.z += az;
  a.gx[i] = gx;
}

__global__ void __launch_bounds__(kAdjBlock) k_adj_xsph(AdjArgs a) {
  if (adj_failed(a.s.status)) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = a.s.n;
  if (i >= n) return;
  const float4* __restrict__ x1 = a.rec.p + static_cast<size_t>(a.iters) * n;
  const float4 xi = x1[i];
  const float4 vi = a.v2[i];
  const SceneConst& c = a.s.sc[__float_as_int(a.rec.p[i].w)];
  const float4 g3 = a.gv3[i];
  float4 gx = a.gx[i];
  float g2x = g3.x, g2y = g3.y, g2z = g3.z, grho = 0.0f;
  if (c.xsph_on) {
    const float ri = a.rec.rho[i];
    const float ai = ri > 0.0f ? c.mass / ri : 0.0f;
    float wsum = 0.0f, vx = 0.0f, vy = 0.0f, vz = 0.0f, rsum = 0.0f;
    auto load = [&](int j) { return Rec3{__ldg(x1 + j), __ldg(a.v2 + j), __ldg(a.gv3 + j)}; };
    for_list_rec(a.s, i, load, [&](const Rec3 rj) {
      const float4 xj = rj.a;
      const float dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
      const float r2 = d2(dx, dy, dz);
      if (!(r2 < c.h2)) return;
      const float4 vj = rj.b;
      const float aj = vj.w;
      const float4 gj = rj.c;
      const float w = Wp(c, r2);
      const float ux = vj.x - vi.x, uy = vj.y - vi.y, uz = vj.z - vi.z;
      const float ti = ux * g3.x + uy * g3.y + uz * g3.z;
      const float tj = -(ux * gj.x + uy * gj.y + uz * gj.z);
      wsum += w * aj;
      vx += w * gj.x;
      vy += w * gj.y;
      vz += w * gj.z;
      const float coef = 2.0f * dW(c, r2) * c.visc_c * (aj * ti + ai * tj);
      gx.x += coef * dx;
      gx.y += coef * dy;
      gx.z += coef * dz;
      rsum += w * tj;
    });
    g2x = g3.x - c.visc_c * wsum * g3.x + c.visc_c * ai * vx;
    g2y = g3.y - c.visc_c * wsum * g3.y + c.visc_c * ai * vy;
    g2z = g3.z - c.visc_c * wsum * g3.z + c.visc_c * ai * vz;
    grho = ri > 0.0f ? -(c.mass / (ri * ri)) * c.visc_c * rsum : 0.0f;
  }
  a.grho[i] = grho;
  // commit: v2 = (p^K - x0)/dt, x1 = p^K
  a.gp[i] = make_float4(gx.x + g2x / c.dt, gx.y + g2y / c.dt, gx.z + g2z / c.dt, 0.0f);
  a.gx0[i] = make_float4(-g2x / c.dt, -g2y / c.dt, -g2z / c.dt, 0.0f);
}

__global__ void __launch_bounds__(kAdjBlock) k_adj_proj(AdjArgs a, int it) {
  if (adj_failed(a.s.status)) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = a.s.n;
  if (i >= n) return;
  const SceneConst& c = a.s.sc[__float_as_int(a.rec.p[i].w)];
  const float4 q0 = a.rec.q[static_cast<size_t>(it) * n + i];
  float q[3] = {q0.x, q0.y, q0.z};
  const float4 gp = a.gp[i];
  float g[3] = {gp.x, gp.y, gp.z};
  unsigned act = 0;
  for (int k = 0; k < c.plane_count; ++k) {
    const float4 pl = c.planes[k];
    const float pen = -plane_sd(pl, q[0], q[1], q[2]);
    if (pen > 0.0f) {
      act |= 1u << k;
      q[0] = __fadd_rn(q[0], __fmul_rn(pl.x, pen));
      q[1] = __fadd_rn(q[1], __fmul_rn(pl.y, pen));
      q[2] = __fadd_rn(q[2], __fmul_rn(pl.z, pen));
    }
  }
  for (int k = c.plane_count - 1; k >= 0; --k) {
    if (!(act >> k & 1u)) continue;
    const float4 pl = c.planes[k];
    const float gn = pl.x * g[0] + pl.y * g[1] + pl.z * g[2];
    g[0] -= gn * pl.x;
    g[1] -= gn * pl.y;
    g[2] -= gn * pl.z;
  }
  a.gd[i] = make_float4(g[0], g[1], g[2], a.rec.lambda[static_cast<size_t>(it) * n + i]);
}

__global__ void __launch_bounds__(kAdjBlock) k_adj_delta(AdjArgs a, int it) {
  if (adj_failed(a.s.status)) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = a.s.n;
  if (i >= n) return;
  const float4* __restrict__ P = a.rec.p + static_cast<size_t>(it) * n;
  const float4* __restrict__ GD = a.gd;  // w = lambda_j
  const float4 pi = P[i];
  const SceneConst& c = a.s.sc[__float_as_int(a.rec.p[i].w)];
  const float4 gdi = GD[i];
  const float li = gdi.w;
  const bool scorr = c.scorr_on != 0;
  float gx = gdi.x, gy = gdi.y, gz = gdi.z, gl = 0.0f;
  float rs = 0.0f, Gx = 0.0f, Gy = 0.0f, Gz = 0.0f, s1 = 0.0f;
  auto load = [&](int j) { return Rec2{__ldg(P + j), __ldg(GD + j)}; };
  for_list_rec(a.s, i, load, [&](const Rec2 rj) {
    const float4 pj = rj.a;
    const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
    const float r2 = d2(dx, dy, dz);
    if (!(r2 < c.h2)) return;
    const bool clamp = r2 < c.min_r2;
    const float r = sqrtf(clamp ? c.min_r2 : r2);
    const float f = Fs(c, r), fpr = clamp ? 0.0f : dFs(c, r) / r;
    float s = li + rj.b.w;
    float alpha;
    if (scorr) {
      const float x = Wp(c, r2) * c.scorr_inv_wdq;
      s += c.scorr_neg_k * powi(x, c.scorr_n);
      alpha = s * fpr + 2.0f * f * c.scorr_neg_k * static_cast<float>(c.scorr_n) * powi(x, c.scorr_n - 1) *
                            c.scorr_inv_wdq * dW(c, r2);
    } else {
      alpha = s * fpr;
    }
    const float4 gdj = rj.b;
    const float ex = gdi.x - gdj.x, ey = gdi.y - gdj.y, ez = gdi.z - gdj.z;
    const float de = dx * ex + dy * ey + dz * ez;
    gx += c.inv_density * (s * f * ex + alpha * de * dx);
    gy += c.inv_density * (s * f * ey + alpha * de * dy);
    gz += c.inv_density * (s * f * ez + alpha * de * dz);
    gl += c.inv_density * f * de;
    rs += Wp(c, r2);
    Gx += f * dx;
    Gy += f * dy;
    Gz += f * dz;
    s1 += f * f * r2;
  });
  const float rho = c.mass * (rs + c.w0);
  const float C = rho * c.inv_density - 1.0f;
  const float S = c.grad_scale * c.grad_scale * (s1 + Gx * Gx + Gy * Gy + Gz * Gz);
  const float lam = -C / (S + c.epsilon);
  const float gC = -gl / (S + c.epsilon);
  const float gS = -gl * lam / (S + c.epsilon);
  a.pg[i] = make_float4(pi.x, pi.y, pi.z, (it == a.iters - 1 ? a.grho[i] : 0.0f) + gC * c.inv_density);
  a.aux[i] = make_float4(Gx, Gy, Gz, gS);
  a.gp[i] = make_float4(gx, gy, gz, 0.0f);
}

__global__ void __launch_bounds__(kAdjBlock) k_adj_lambda(AdjArgs a, int it) {
  if (adj_failed(a.s.status)) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = a.s.n;
  if (i >= n) return;
  const float4* __restrict__ PG = a.pg;  // (p_j, dL/drho_j)
  const float4* __restrict__ AUX = a.aux;
  const float4 pgi = PG[i];
  const SceneConst& c = a.s.sc[__float_as_int(a.rec.p[i].w)];
  const float4 ai = AUX[i];
  const float gri = pgi.w;
  const float gs2 = c.grad_scale * c.grad_scale;
  float ax = 0.0f, ay = 0.0f, az = 0.0f;
  auto load = [&](int j) { return Rec2{__ldg(PG + j), __ldg(AUX + j)}; };
  for_list_rec(a.s, i, load, [&](const Rec2 rj) {
    const float4 pj = rj.a;
    const float dx = pgi.x - pj.x, dy = pgi.y - pj.y, dz = pgi.z - pj.z;
    const float r2 = d2(dx, dy, dz);
    if (!(r2 < c.h2)) return;
    const bool clamp = r2 < c.min_r2;
    const float r = sqrtf(clamp ? c.min_r2 : r2);
    const float f = Fs(c, r), fpr = clamp ? 0.0f : dFs(c, r) / r;
    const float4 aj = rj.b;
    const float grj = pj.w;
    const float dGi = dx * ai.x + dy * ai.y + dz * ai.z;
    const float dGj = dx * aj.x + dy * aj.y + dz * aj.z;
    const float t = 2.0f * c.mass * dW(c, r2) * (gri + grj) +
                    gs2 * (ai.w + aj.w) * (2.0f * f * fpr * r2 + 2.0f * f * f) +
                    2.0f * gs2 * fpr * (ai.w * dGi - aj.w * dGj);
    const float u = 2.0f * f * gs2;
    ax += t * dx + u * (ai.w * ai.x - aj.w * aj.x);
    ay += t * dy + u * (ai.w * ai.y - aj.w * aj.y);
    az += t * dz + u * (ai.w * ai.z - aj.w * aj.z);
  });
  float4 g = a.gp[i];
  g.x += ax;
  g.y += ay;
  g.z += az;
  a.gp[i] = g;
}

__global__ void __launch_bounds__(kAdjBlock) k_adj_in(AdjArgs a) {
  if (adj_failed(a.s.status)) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = a.s.n;
  if (i >= n) return;
  const SceneConst& c = a.s.sc[__float_as_int(a.rec.p[i].w)];
  const int o = __float_as_int(a.rec.x0[i].w);
  const float4 gp = a.gp[i];
  const float4 g0 = a.gx0[i];
  a.g_pos_in[o] = g0.x + gp.x;
  a.g_pos_in[n + o] = g0.y + gp.y;
  a.g_pos_in[2 * n + o] = g0.z + gp.z;
  a.g_vel_in[o] = gp.x * c.dt;
  a.g_vel_in[n + o] = gp.y * c.dt;
  a.g_vel_in[2 * n + o] = gp.z * c.dt;
}

}  // namespace

cudaError_t enqueue_adjoint(const AdjArgs& a, cudaStream_t st) {
  const int nb = (a.s.n + kAdjBlock - 1) / kAdjBlock;
  if (a.s.n == 0) return cudaSuccess;
  k_adj_prepare<<<nb, kAdjBlock, 0, st>>>(a);
  k_adj_out<<<nb, kAdjBlock, 0, st>>>(a);
  if (a.vorticity) {
    k_adj_eta<<<nb, kAdjBlock, 0, st>>>(a);
    k_adj_omega<<<nb, kAdjBlock, 0, st>>>(a);
  }
  k_adj_xsph<<<nb, kAdjBlock, 0, st>>>(a);
  for (int it = a.iters - 1; it >= 0; --it) {
    k_adj_proj<<<nb, kAdjBlock, 0, st>>>(a, it);
    k_adj_delta<<<nb, kAdjBlock, 0, st>>>(a, it);
    k_adj_lambda<<<nb, kAdjBlock, 0, st>>>(a, it);
  }
  k_adj_in<<<nb, kAdjBlock, 0, st>>>(a);
  return cudaGetLastError();
}

}  // namespace fgb
