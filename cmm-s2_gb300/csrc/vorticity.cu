// Vorticity at the back-traced sample points (sm_103a):
//   omega = omega0(X) + 2 Omega cos(theta(X)) - 2 Omega cos(theta_grid)
// (cmm_s2/core/spherical_simulations.py:269-272), with omega0 one of the
// barotropic fields of cmm_s2/core/dynamical_fields.py:181-214 or the
// synthetic benchmark fields, optionally plus a real spherical-harmonic
// series.
#include <cuda_runtime.h>

#include "cmm_internal.h"
#include "device_common.cuh"

namespace cmm {

using namespace dev;

namespace {

constexpr double kPi = 3.141592653589793;

struct VortParams {
  int kind;
  double p[12];
};

// zonal jet family (dynamical_fields.py:181-192)
__device__ __forceinline__ double jet(double theta, double theta_c) {
  const double beta2 = 144.0;
  const double u_lt = (kPi / 2) * exp(-2 * beta2 * (1 - cos(-theta + kPi / 2 - theta_c)));
  return (cos(-theta + kPi / 2) * (2 * beta2 * (cos(theta_c) * sin(-theta + kPi / 2) -
                                                sin(theta_c) * cos(-theta + kPi / 2))) +
          sin(kPi / 2 - theta)) *
         u_lt;
}

__device__ double omega0(const VortParams& v, double phi, double theta) {
  switch (v.kind) {
    case CMM_VORT_ROSSBY_HAURWITZ: {  // dynamical_fields.py:205-210
      const double alpha = 1.0 / 30.0, Omega = 2 * kPi;
      const double s = sin(theta);
      return 30 * cos(theta) * cos(4 * (phi + 2 * Omega * alpha * v.p[0])) * (s * s * s * s);
    }
    case CMM_VORT_ZONAL_JET:
      return jet(theta, kPi / 4);
    case CMM_VORT_PERTURBED_JET:
      return jet(theta, kPi / 4 + 0.01 * cos(12 * phi));
    case CMM_VORT_MULTI_JET:
      return jet(theta, kPi / 4 + 0.01 * cos(12 * phi)) +
             jet(theta - kPi / 8, kPi / 4 + 0.01 * cos(12 * phi));
    case CMM_VORT_GAUSSIAN_VORTEX: {  // dynamical_fields.py:200-203
      const double x = sin(theta) * cos(phi), y = sin(theta) * sin(phi), z = cos(theta);
      return 4 * kPi * exp(-((x - 1) * (x - 1) + y * y + z * z) / (1.0 / 16.0));
    }
    case CMM_VORT_PERTURBED_RH: {  // dynamical_fields.py:213-215
      const double s = sin(theta);
      return 30 * cos(theta) * cos(4 * phi) * (s * s * s * s) + 0.1 * sin(theta) * cos(30 * theta);
    }
    case CMM_VORT_GAUSSIAN_JETS: {  // p = amplitude, width, n, lat_1..lat_n
      const double lat = kPi / 2 - theta;
      double s = 0.0;
      const int n = (int)v.p[2];
      for (int j = 0; j < n && j < 9; ++j) {
        const double d = (lat - v.p[3 + j]) / v.p[1];
        s += v.p[0] * exp(-d * d);
      }
      return s;
    }
    default:
      return 0.0;
  }
}

// The same fields in FP32 (mixed form, velmesh field32): angles from atan2f
// and FP32 elementary functions; relative error ~1e-7, below the mixed
// form's transform error (~1e-5).
__device__ float jet_f(float theta, float theta_c) {
  const float pi = 3.14159265358979f, beta2 = 144.0f;
  const float u_lt = (pi / 2) * expf(-2 * beta2 * (1 - cosf(-theta + pi / 2 - theta_c)));
  return (cosf(-theta + pi / 2) * (2 * beta2 * (cosf(theta_c) * sinf(-theta + pi / 2) -
                                                sinf(theta_c) * cosf(-theta + pi / 2))) +
          sinf(pi / 2 - theta)) *
         u_lt;
}

__device__ float omega0_f(const VortParams& v, float phi, float theta) {
  const float pi = 3.14159265358979f;
  switch (v.kind) {
    case CMM_VORT_ROSSBY_HAURWITZ: {
      const float alpha = 1.0f / 30.0f, Omega = 2 * pi;
      const float s = sinf(theta);
      return 30 * cosf(theta) * cosf(4 * (phi + 2 * Omega * alpha * (float)v.p[0])) * (s * s * s * s);
    }
    case CMM_VORT_ZONAL_JET:
      return jet_f(theta, pi / 4);
    case CMM_VORT_PERTURBED_JET:
      return jet_f(theta, pi / 4 + 0.01f * cosf(12 * phi));
    case CMM_VORT_MULTI_JET:
      return jet_f(theta, pi / 4 + 0.01f * cosf(12 * phi)) + jet_f(theta - pi / 8, pi / 4 + 0.01f * cosf(12 * phi));
    case CMM_VORT_GAUSSIAN_VORTEX: {
      const float x = sinf(theta) * cosf(phi), y = sinf(theta) * sinf(phi), z = cosf(theta);
      return 4 * pi * expf(-((x - 1) * (x - 1) + y * y + z * z) / (1.0f / 16.0f));
    }
    case CMM_VORT_PERTURBED_RH: {
      const float s = sinf(theta);
      return 30 * cosf(theta) * cosf(4 * phi) * (s * s * s * s) + 0.1f * sinf(theta) * cosf(30 * theta);
    }
    case CMM_VORT_GAUSSIAN_JETS: {
      const float lat = pi / 2 - theta;
      float s = 0.0f;
      const int n = (int)v.p[2];
      for (int j = 0; j < n && j < 9; ++j) {
        const float d = (lat - (float)v.p[3 + j]) / (float)v.p[1];
        s += (float)v.p[0] * expf(-d * d);
      }
      return s;
    }
    default:
      return 0.0f;
  }
}

__global__ void __launch_bounds__(256) vorticity_kernel(VortParams vp, const double* __restrict__ sh, int lmax,
                                 MeshView vm, const double* __restrict__ spline, double rot,
                                 const double* __restrict__ X, int64_t Q, int npr,
                                 const double* __restrict__ cos_ring, double* __restrict__ omega) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < Q;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double x = X[3 * i], y = X[3 * i + 1], z = X[3 * i + 2];
    double w = 0.0, ct;
    if (vm.field32) {
      const float xf = to_f32_trunc(x), yf = to_f32_trunc(y), zf = to_f32_trunc(z);
      float phif = atan2f(yf, xf);
      if (phif < 0.f) phif += 6.28318530717958647692f;
      const float thf = atan2f(sqrtf(xf * xf + yf * yf), zf);
      if (vp.kind != CMM_VORT_NONE) w = (double)omega0_f(vp, phif, thf);
      ct = z * rsqrt(x * x + y * y + z * z);   // cos(theta), FP64
    } else if (vp.kind != CMM_VORT_NONE) {
      double phi, theta;
      cart2sphere(x, y, z, &phi, &theta);
      w = omega0(vp, phi, theta);
      ct = cos(theta);
    } else {
      ct = z * rsqrt(x * x + y * y + z * z);
    }
    if (sh) {
      double v;
      sh_series_n<1>(vm, sh, lmax, sh_point(x, y, z), &v);
      w += v;
    }
    if (spline) w += (vm.field32 && vm.tri_loc_f) ? latlon_scalar_f(vm, spline, x, y, z)
                                                  : latlon_scalar(vm, spline, x, y, z);
    const double r = w + 2 * rot * ct - 2 * rot * cos_ring[i / npr];
    if (!isfinite(r)) atomicOr(vm.status, CMM_FLAG_NONFINITE);
    omega[i] = r;
  }
}

}  // namespace

int launch_vorticity(int kind, const double* params, int nparams, const double* sh, int lmax,
                     const MeshView& vm, const double* spline, double rot, const double* X,
                     int64_t Q, int npr, const double* cos_ring, double* omega, cudaStream_t s) {
  VortParams vp{};
  vp.kind = kind;
  for (int k = 0; k < nparams && k < 12; ++k) vp.p[k] = params[k];
  const int b = block_for(vm, kTuneVorticity, 128, Q);
  vorticity_kernel<<<grid_for(Q, b), b, 0, s>>>(vp, sh, lmax, vm, spline, rot, X, Q, npr,
                                                    cos_ring, omega);
  note_launch();
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? CMM_OK : cuda_fail(e, "vorticity_kernel");
}

}  // namespace cmm
