// Backward integrators with projection onto the sphere after each stage
// (cmm_s2/core/evolution_functions.py:19-85), shared by the spline velocity
// (velocity.cu) and the analytic transport flows (transport.cu).  The
// velocity source is a functor vel(stage, x, y, z, V) whose stage k is the
// scheme's k-th evaluation time, in the order the reference calls V:
//   CMM_EULER          t
//   CMM_IMPROVED_EULER t, t+dt
//   CMM_RK4            t+dt, t+dt/2, t+dt/2, t
//   CMM_RK2            t+dt, t+dt/2
#pragma once

#include <cuda_runtime.h>

#include "cmm_gpu.h"

namespace cmm {
namespace dev {

// div_norm (evolution_functions.py:82-85): x * (1 / |x|), the reciprocal
// norm from the FP64 rsqrt (within 1 ulp): an IEEE square root and division
// cost ~25 FP64-pipe instructions, a fifth of the RK4 foot point's FP64
// budget on GB300.
__device__ __forceinline__ void sphere_proj(double* x) {
  const double r = rsqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
  x[0] *= r;
  x[1] *= r;
  x[2] *= r;
}

template <class Vel>
__device__ __forceinline__ void integrate_back(const Vel& vel, int scheme, double dt, double* x) {
  double v1[3], v2[3], s[3];
  vel(0, x[0], x[1], x[2], v1);
  if (scheme == CMM_EULER) {
    for (int c = 0; c < 3; ++c) x[c] = x[c] - dt * v1[c];
    sphere_proj(x);
    return;
  }
  if (scheme == CMM_IMPROVED_EULER) {
    for (int c = 0; c < 3; ++c) s[c] = x[c] - dt * v1[c];
    sphere_proj(s);
    vel(1, s[0], s[1], s[2], v2);
    for (int c = 0; c < 3; ++c) x[c] = x[c] - (dt / 2) * (v1[c] + v2[c]);
    sphere_proj(x);
    return;
  }
  if (scheme == CMM_RK2) {  // RK2_proj, :68-78
    for (int c = 0; c < 3; ++c) s[c] = x[c] - (dt / 2) * v1[c];
    sphere_proj(s);
    vel(1, s[0], s[1], s[2], v2);
    for (int c = 0; c < 3; ++c) x[c] = x[c] - dt * v2[c];
    sphere_proj(x);
    return;
  }
  double v3[3], v4[3];
  for (int c = 0; c < 3; ++c) s[c] = x[c] - dt * v1[c] / 2;
  sphere_proj(s);
  vel(1, s[0], s[1], s[2], v2);
  for (int c = 0; c < 3; ++c) s[c] = x[c] - (dt / 2) * v2[c];
  sphere_proj(s);
  vel(2, s[0], s[1], s[2], v3);
  for (int c = 0; c < 3; ++c) s[c] = x[c] - dt * v3[c];
  sphere_proj(s);
  vel(3, s[0], s[1], s[2], v4);
  for (int c = 0; c < 3; ++c) x[c] = x[c] - (dt / 6) * (v1[c] + 2 * v2[c] + 2 * v3[c] + v4[c]);
  sphere_proj(x);
}

}  // namespace dev
}  // namespace cmm
