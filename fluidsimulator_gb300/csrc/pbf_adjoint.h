// Launch interface of the adjoint kernels (pbf_adjoint.cu).
#pragma once

#include <cuda_runtime.h>

#include "pbf_common.cuh"
#include "pbf_launch.h"

namespace fgb {

struct AdjArgs {
  StepArgs s;        // the recorded step: lists, scene constants, status
  StepRecord rec;    // its internals
  int iters;
  float4* v2;        // committed velocity
  float4* gx;        // cotangent of the committed positions (accumulates)
  float4* gv;        // cotangent of the output velocity
  float4* gv3;       // ... before restitution
  float4* gp;        // cotangent of p^k
  float4* gd;        // cotangent of the correction of iteration k; w = lambda_i^k
  float4* gx0;       // cotangent of the input positions through the commit
  float4* aux;       // (G_i, dL/dS_i) of the density constraint
  float4* pg;        // (p_i of the iteration reversed, dL/drho_i total)
  float* grho;       // dL/drho_i from XSPH
  float* cc;         // per-particle share of dL/dc (XSPH coefficient)
  int vorticity;     // some scene runs vorticity confinement
  float4* v3;        // velocity after XSPH (recomputed)
  float4* dv;        // XSPH sum (recomputed)
  float4* gv4;       // cotangent of the velocity after vorticity, before restitution
  float4* eb;        // cotangent of eta
  float4* obd;       // cotangent of omega through the confinement force
  float4* ob;        // cotangent of omega (total)
  const float* g_pos_out;  // caller order, 3n floats: x block, y block, z block
  const float* g_vel_out;
  float* g_pos_in;
  float* g_vel_in;
};

cudaError_t enqueue_adjoint(const AdjArgs& a, cudaStream_t stream);

}  // namespace fgb
