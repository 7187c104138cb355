// Linear transport on the sphere with the reference's analytic test flows
// and tracer fields (sm_103a): the velocity fields of
// cmm_s2/core/dynamical_fields.py:18-107 evaluated in closed form inside
// the backward integrators, so the CMM map update of
// cmm_s2/tests/test_spherical_transport.py (advect_project_sphere with
// U = u_deform_rot, ...) runs without a velocity mesh; and the tracer
// initial conditions (:85-159, and the smooth test function of
// tests/test_spherical_transport.py:36-38) evaluated at composed points.
//
// Time-dependent rotation matrices and cos(pi t / T) factors are computed
// on the host once per stage time (FlowSpec), in FP64 with the reference's
// formulas; the kernels see only products and sums.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <mutex>

#include "cmm_internal.h"
#include "device_common.cuh"
#include "integrators.cuh"

namespace cmm {

using namespace dev;

namespace {

constexpr int kBlock = 128;
constexpr double kPi = 3.141592653589793;
constexpr double kRho0 = 3.0;  // rho_0, dynamical_fields.py:44

struct FlowStage {
  double fwd[9];   // rotation into the moving frame
  double back[9];  // rotation back
  double c1;       // 2 k cos(pi t / T), k = 2 (u_deform)
  double cdiv;     // cos(pi t / T) (u_div)
};

struct FlowSpec {
  int kind;
  double wx, wz;   // solid-body rotation vector (c sin(alpha), 0, c cos(alpha)), c = -2 pi / T
  FlowStage st[4];
};

__device__ __forceinline__ void rotate3(const double* L, double x, double y, double z, double* o) {
  o[0] = L[0] * x + L[1] * y + L[2] * z;
  o[1] = L[3] * x + L[4] * y + L[5] * z;
  o[2] = L[6] * x + L[7] * y + L[8] * z;
}

// utils.cross(a, b) with b = (bx, by, bz)
__device__ __forceinline__ void cross3(double ax, double ay, double az, double bx, double by, double bz,
                                       double* o) {
  o[0] = ay * bz - az * by;
  o[1] = az * bx - ax * bz;
  o[2] = ax * by - ay * bx;
}

__device__ __forceinline__ void u_sbr(const FlowSpec& f, double x, double y, double z, double* V) {
  cross3(x, y, z, f.wx, 0.0, f.wz, V);  // :18-22
}

__device__ __forceinline__ void u_deform(double c1, double x, double y, double z, double* V) {
  cross3(x, y, z, 0.0 * x, c1 * y, 0.0 * z, V);  // :24-30
}

// omega_r (:48-55): angular speed of the static vortex at colatitude theta
__device__ __forceinline__ double omega_r(double theta) {
  if (theta == 0.0) return 0.0;
  const double c = sin(theta);
  const double a = kRho0 * c;
  const double sech = 1.0 / cosh(a);
  return (2 * kPi) * sqrt(3.0) * (3.0 / 2.0) * (1.0 / a) * tanh(a) * (sech * sech);
}

__device__ __forceinline__ void u_static_vortex(double x, double y, double z, double* V) {
  double phi, theta;  // :57-65
  cart2sphere(x, y, z, &phi, &theta);
  const double w = omega_r(theta);
  V[0] = -y * w;
  V[1] = x * w;
  V[2] = 0.0 * z;
}

// tan_proj (utils.py:29-34)
__device__ __forceinline__ void tan_proj(double x, double y, double z, const double* A, double* o) {
  o[0] = (1 - x * x) * A[0] + (-x * y) * A[1] + (-x * z) * A[2];
  o[1] = (-x * y) * A[0] + (1 - y * y) * A[1] + (-y * z) * A[2];
  o[2] = (-x * z) * A[0] + (-y * z) * A[1] + (1 - z * z) * A[2];
}

__device__ void flow_at(const FlowSpec& f, int s, double x, double y, double z, double* V) {
  const FlowStage& g = f.st[s];
  switch (f.kind) {
    case CMM_FLOW_SOLID_BODY:
      u_sbr(f, x, y, z, V);
      return;
    case CMM_FLOW_DEFORM:
      u_deform(g.c1, x, y, z, V);
      return;
    case CMM_FLOW_DEFORM_ROT: {  // :32-42
      double r[3], u[3], w[3];
      rotate3(g.fwd, x, y, z, r);
      u_deform(g.c1, r[0], r[1], r[2], u);
      rotate3(g.back, u[0], u[1], u[2], w);
      u_sbr(f, x, y, z, V);
      V[0] = w[0] + V[0];
      V[1] = w[1] + V[1];
      V[2] = w[2] + V[2];
      return;
    }
    case CMM_FLOW_STATIC_VORTEX:
      u_static_vortex(x, y, z, V);
      return;
    case CMM_FLOW_ROTATING_VORTEX:  // :67-76
    case CMM_FLOW_EQUATOR_VORTEX: {  // :78-83
      double r[3], u[3], w[3];
      rotate3(g.fwd, x, y, z, r);
      u_static_vortex(r[0], r[1], r[2], u);
      rotate3(g.back, u[0], u[1], u[2], w);
      if (f.kind == CMM_FLOW_EQUATOR_VORTEX) {
        V[0] = w[0];
        V[1] = w[1];
        V[2] = w[2];
        return;
      }
      u_sbr(f, x, y, z, V);
      V[0] = w[0] + V[0];
      V[1] = w[1] + V[1];
      V[2] = w[2] + V[2];
      return;
    }
    case CMM_FLOW_DIVERGENT: {  // :97-107
      double phi, theta;
      cart2sphere(x, y, z, &phi, &theta);
      const double sp2 = sin(phi / 2), st = sin(theta), ct = cos(theta), sph = sin(phi), cph = cos(phi);
      const double u = -(sp2 * sp2) * sin(2 * theta) * st * g.cdiv;
      const double v = (-0.5) * sph * (st * st * st) * g.cdiv;
      const double A[3] = {ct * cph * v - st * sph * u, ct * sph * v + st * cph * u, -st * v};
      tan_proj(x, y, z, A, V);
      return;
    }
    default:
      V[0] = V[1] = V[2] = 0.0;
  }
}

struct FlowVel {
  const FlowSpec& f;
  __device__ __forceinline__ void operator()(int s, double x, double y, double z, double* V) const {
    flow_at(f, s, x, y, z, V);
  }
};

// x, out: (3,n) component-major
__global__ void __launch_bounds__(kBlock) flow_velocity_kernel(MeshView m, FlowSpec f,
                                                               const double* __restrict__ x, int64_t n,
                                                               double* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double px = x[i], py = x[n + i], pz = x[2 * n + i];
    double V[3] = {nan(""), nan(""), nan("")};
    if (finite3(px, py, pz))
      flow_at(f, 0, px, py, pz, V);
    if (!finite3(V[0], V[1], V[2])) flag(m, CMM_FLAG_NONFINITE);
    out[i] = V[0];
    out[n + i] = V[1];
    out[2 * n + i] = V[2];
  }
}

__global__ void __launch_bounds__(kBlock) flow_integrate_kernel(MeshView m, FlowSpec f, int scheme, double dt,
                                                                const double* __restrict__ x, int64_t n,
                                                                double* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double p[3] = {x[i], x[n + i], x[2 * n + i]};
    if (finite3(p[0], p[1], p[2])) integrate_back(FlowVel{f}, scheme, dt, p);
    if (!finite3(p[0], p[1], p[2])) flag(m, CMM_FLAG_NONFINITE);
    out[i] = p[0];
    out[n + i] = p[1];
    out[2 * n + i] = p[2];
  }
}

// Foot points of the vertices and stencil points (advect,
// evolution_functions.py:117-133), the layout of advect_points_kernel:
// work = yn (3,nv) followed by the stencil foot points (3,4,nv).
__global__ void __launch_bounds__(kBlock) flow_advect_points_kernel(MeshView mesh, FlowSpec f, int scheme,
                                                                    double dt, const double* __restrict__ s_pts,
                                                                    double* __restrict__ work) {
  const int64_t nv = mesh.nv, n = 5 * nv;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double p[3];
    const int64_t j = i - nv;
    if (i < nv) {
      p[0] = mesh.verts[4 * i];
      p[1] = mesh.verts[4 * i + 1];
      p[2] = mesh.verts[4 * i + 2];
    } else {
      p[0] = s_pts[j];
      p[1] = s_pts[4 * nv + j];
      p[2] = s_pts[8 * nv + j];
    }
    integrate_back(FlowVel{f}, scheme, dt, p);
    if (!finite3(p[0], p[1], p[2])) flag(mesh, CMM_FLAG_NONFINITE);
    if (i < nv) {
      work[i] = p[0];
      work[nv + i] = p[1];
      work[2 * nv + i] = p[2];
    } else {
      double* sn = work + 3 * nv;
      sn[j] = p[0];
      sn[4 * nv + j] = p[1];
      sn[8 * nv + j] = p[2];
    }
  }
}

// ----------------------------------------------------------------- tracers
struct TracerSpec {
  int kind;
  double t;
  double rot[9];   // rotating_vort_IC: Rot_x(pi/2) Rot_z(0)^T
};

// great-circle distance of (phi, theta) to a bell centre (:124-127)
__device__ __forceinline__ double bell_r(double phi, double theta, double phic, double thec) {
  const double arg = sin(thec - kPi / 2) * sin(theta - kPi / 2) +
                     cos(thec - kPi / 2) * cos(theta - kPi / 2) * cos(phi - phic);
  return acos(arg);  // NaN outside [-1, 1], as numpy's arccos; NaN < R is false
}

__device__ double tracer_at(const TracerSpec& ts, double x, double y, double z) {
  const double phic1 = kPi + kPi / 6, phic2 = kPi - kPi / 6, thec = kPi / 2, R = 0.5, h0 = 1.0;
  switch (ts.kind) {
    case CMM_TRACER_COSINE_BELL: {  // :122-137
      double phi, theta;
      cart2sphere(x, y, z, &phi, &theta);
      const double r1 = bell_r(phi, theta, phic1, thec), r2 = bell_r(phi, theta, phic2, thec);
      const double o1 = r1 < R ? (h0 / 2) * (1 + cos(r1 * kPi / R)) : 0.0;
      const double o2 = r2 < R ? (h0 / 2) * (1 + cos(r2 * kPi / R)) : 0.0;
      return 0.9 * (o1 + o2) + 0.1;
    }
    case CMM_TRACER_SLOTTED_CYLINDERS: {  // :139-157
      double phi, theta;
      cart2sphere(x, y, z, &phi, &theta);
      const double r1 = bell_r(phi, theta, phic1, thec), r2 = bell_r(phi, theta, phic2, thec);
      double o1 = 0.0, o2 = 0.0;
      if (r1 <= R && fabs(phi - phic1) >= R / 6) o1 = 0.9;
      if (r1 <= R && fabs(phi - phic1) < R / 6 && theta < (-5 * R / 12 + kPi / 2)) o1 = 0.9;
      if (r2 <= R && fabs(phi - phic2) >= R / 6) o2 = 0.9;
      if (r2 <= R && fabs(phi - phic2) < R / 6 && theta > (5 * R / 12 + kPi / 2)) o2 = 0.9;
      return o1 + o2 + 0.1;
    }
    case CMM_TRACER_STATIC_VORTEX:      // static_vort_IC, :85-88
    case CMM_TRACER_ROTATING_VORTEX: {  // rotating_vort_IC, :90-95
      double p[3] = {x, y, z};
      if (ts.kind == CMM_TRACER_ROTATING_VORTEX) rotate3(ts.rot, x, y, z, p);
      double phi, theta;
      cart2sphere(p[0], p[1], p[2], &phi, &theta);
      const double rho = kRho0 * sin(theta);
      return 1 - tanh((rho / 5) * sin(phi - omega_r(theta) * ts.t));
    }
    case CMM_TRACER_SMOOTH_TEST: {  // tests/test_spherical_transport.py:36-38
      const double y7 = y * y * y * y * y * y * y, z5 = z * z * z * z * z;
      return sin(x * x) * (10 * cos(y - 2)) + cos(10 * z5) + 2 * sin(x * 3 * (z - 0.1) + y7);
    }
    default:
      return 0.0;
  }
}

// random_initial_condition (:158-172): sum over 1 <= l <= 32, -l <= m < l
// of c_lm Re Y_l^m(phi, theta), c the first 1056 of numpy's legacy
// uniform(-1, 1, 33^2) draws after seed(42).  Re Y_l^-m = (-1)^m Re Y_l^m,
// so the field is a cosine series sum_{m>=0} cos(m phi) sum_l A_lm Pbar_lm
// (orthonormal Pbar with the Condon-Shortley phase, as scipy's sph_harm).
// Tables [m][l] in constant memory: every lane reads the same entry.
constexpr int kRandL = 32, kRandW = kRandL + 1;
__constant__ double c_rand_A[kRandW * kRandW];       // A_lm at [m][l]
__constant__ double c_rand_ab[2 * kRandW * kRandW];  // (a_lm, 1 / a_{l-1,m}) at [m][l]
__constant__ double c_rand_fm[kRandW];               // sqrt((2m+1)/(2m))

__device__ double random_sh_at(double x, double y, double z) {
  const ShPoint pt = sh_point(x, y, z);
  double f = 0.0, pmm = 0.28209479177387814;  // sqrt(1/(4 pi))
  double cm = 1.0, sm = 0.0;
  for (int m = 0; m <= kRandL; ++m) {
    if (m > 0) {
      pmm = -pmm * c_rand_fm[m] * pt.st;
      const double c2 = cm * pt.cp - sm * pt.sp;
      sm = sm * pt.cp + cm * pt.sp;
      cm = c2;
    }
    const double* A = c_rand_A + m * kRandW;
    const double* ab = c_rand_ab + 2 * m * kRandW;
    double p1 = 0.0, p = pmm, acc = A[m] * pmm;
    for (int l = m + 1; l <= kRandL; ++l) {
      const double pn = ab[2 * l] * (pt.ct * p - ab[2 * l + 1] * p1);
      p1 = p;
      p = pn;
      acc += A[l] * p;
    }
    f += acc * cm;
  }
  return f;
}

// X (n,3) points -> out (n,)
__global__ void __launch_bounds__(kBlock) tracer_kernel(MeshView m, TracerSpec ts, const double* __restrict__ X,
                                                        int64_t n, double* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double x = X[3 * i], y = X[3 * i + 1], z = X[3 * i + 2];
    double v = nan("");
    if (finite3(x, y, z)) v = ts.kind == CMM_TRACER_RANDOM_SH ? random_sh_at(x, y, z) : tracer_at(ts, x, y, z);
    if (!isfinite(v)) flag(m, CMM_FLAG_NONFINITE);
    out[i] = v;
  }
}

// ------------------------------------------------------------------ host
// utils.Rot_x/Rot_y/Rot_z (utils.py:109-116), row-major
void rot_x(double a, double* R) {
  const double c = std::cos(a), s = std::sin(a);
  const double M[9] = {1, 0, 0, 0, c, -s, 0, s, c};
  for (int k = 0; k < 9; ++k) R[k] = M[k];
}
void rot_y(double a, double* R) {
  const double c = std::cos(a), s = std::sin(a);
  const double M[9] = {c, 0, -s, 0, 1, 0, s, 0, c};
  for (int k = 0; k < 9; ++k) R[k] = M[k];
}
void rot_z(double a, double* R) {
  const double c = std::cos(a), s = std::sin(a);
  const double M[9] = {c, -s, 0, s, c, 0, 0, 0, 1};
  for (int k = 0; k < 9; ++k) R[k] = M[k];
}
void transpose3(const double* A, double* T) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) T[3 * j + i] = A[3 * i + j];
}
void matmul3(const double* A, const double* B, double* C) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) C[3 * i + j] = A[3 * i] * B[j] + A[3 * i + 1] * B[3 + j] + A[3 * i + 2] * B[6 + j];
}

void stage_setup(int kind, double T, double alpha, double t, FlowStage* g) {
  g->c1 = 2 * 2 * std::cos(kPi * t / T);
  g->cdiv = std::cos(kPi * t / T);
  double A[9], B[9], At[9], Bt[9];
  for (int k = 0; k < 9; ++k) g->fwd[k] = g->back[k] = k % 4 == 0 ? 1.0 : 0.0;
  if (kind == CMM_FLOW_DEFORM_ROT) {  // tau = 2 pi t
    rot_z(2 * kPi * t, A);
    rot_y(alpha, B);
    transpose3(A, At);
    transpose3(B, Bt);
    matmul3(At, B, g->fwd);
    matmul3(Bt, A, g->back);
  } else if (kind == CMM_FLOW_ROTATING_VORTEX) {  // tau = 2 pi t / T
    rot_x(kPi / 2, A);
    rot_z(2 * kPi * t / T, B);
    transpose3(A, At);
    transpose3(B, Bt);
    matmul3(A, Bt, g->fwd);
    matmul3(B, At, g->back);
  } else if (kind == CMM_FLOW_EQUATOR_VORTEX) {
    rot_x(kPi / 2, A);
    for (int k = 0; k < 9; ++k) g->fwd[k] = A[k];
    transpose3(A, g->back);
  }
}

int make_spec(int kind, double T, double alpha, int scheme, double t, double dt, FlowSpec* f);
int check_launch(const char* what);

}  // namespace

// stage times of each scheme, in the order the integrators call V
// (evolution_functions.py:19-80); 0 for an unknown scheme
int stage_times(int scheme, double t, double dt, double* times) {
  switch (scheme) {
    case CMM_EULER:
      times[0] = t;
      return 1;
    case CMM_IMPROVED_EULER:
      times[0] = t;
      times[1] = t + dt;
      return 2;
    case CMM_RK4:
      times[0] = t + dt;
      times[1] = t + dt / 2;
      times[2] = t + 0.5 * dt;
      times[3] = t;
      return 4;
    case CMM_RK2:
      times[0] = t + dt;
      times[1] = t + dt / 2;
      return 2;
    default:
      return 0;
  }
}

namespace {

int make_spec(int kind, double T, double alpha, int scheme, double t, double dt, FlowSpec* f) {
  if (kind < CMM_FLOW_SOLID_BODY || kind > CMM_FLOW_DIVERGENT) {
    set_last_error("unknown transport flow");
    return CMM_ERR_ARG;
  }
  if (!(T != 0.0) || !std::isfinite(T) || !std::isfinite(alpha)) {
    set_last_error("transport flow: period T must be finite and nonzero, alpha finite");
    return CMM_ERR_ARG;
  }
  double times[4];
  const int nt = scheme < 0 ? 1 : stage_times(scheme, t, dt, times);
  if (scheme < 0) times[0] = t;
  if (nt == 0) {
    set_last_error("unknown integration scheme");
    return CMM_ERR_ARG;
  }
  *f = FlowSpec{};
  f->kind = kind;
  const double c = -2 * kPi / T;
  f->wx = c * std::sin(alpha);
  f->wz = c * std::cos(alpha);
  for (int s = 0; s < nt; ++s) stage_setup(kind, T, alpha, times[s], &f->st[s]);
  return CMM_OK;
}

int check_launch(const char* what) {
  note_launch();
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? CMM_OK : cuda_fail(e, what);
}

}  // namespace

int flow_velocity(const MeshView& m, int kind, double T, double alpha, double t, const double* x, int64_t n,
                  double* out, cudaStream_t s) {
  FlowSpec f;
  int rc = make_spec(kind, T, alpha, -1, t, 0.0, &f);
  if (rc || n == 0) return rc;
  flow_velocity_kernel<<<grid_for(n, kBlock), kBlock, 0, s>>>(m, f, x, n, out);
  return check_launch("flow_velocity_kernel");
}

int flow_integrate(const MeshView& m, int kind, double T, double alpha, int scheme, double t, double dt,
                   const double* x, int64_t n, double* out, cudaStream_t s) {
  FlowSpec f;
  int rc = make_spec(kind, T, alpha, scheme, t, dt, &f);
  if (rc || n == 0) return rc;
  flow_integrate_kernel<<<grid_for(n, kBlock), kBlock, 0, s>>>(m, f, scheme, dt, x, n, out);
  return check_launch("flow_integrate_kernel");
}

int flow_advect_points(const MeshView& mesh, int kind, double T, double alpha, int scheme, double t, double dt,
                       const double* s_pts, double* work, cudaStream_t s) {
  FlowSpec f;
  int rc = make_spec(kind, T, alpha, scheme, t, dt, &f);
  if (rc) return rc;
  const int64_t n = 5LL * mesh.nv;
  const int b = small_block(n, kBlock);
  flow_advect_points_kernel<<<grid_for(n, b), b, 0, s>>>(mesh, f, scheme, dt, s_pts, work);
  return check_launch("flow_advect_points_kernel");
}

namespace {

// MT19937 (Matsumoto & Nishimura 1998) seeded by init_genrand, and the
// 53-bit double of numpy's legacy random_sample ((a >> 5) 2^26 + (b >> 6))
// / 2^53: the generator behind np.random.seed(42); np.random.uniform.
class Mt19937 {
 public:
  explicit Mt19937(uint32_t seed) {
    s_[0] = seed;
    for (int i = 1; i < kN; ++i) s_[i] = 1812433253u * (s_[i - 1] ^ (s_[i - 1] >> 30)) + (uint32_t)i;
  }
  uint32_t next() {
    if (i_ >= kN) {
      for (int k = 0; k < kN; ++k) {
        const uint32_t y = (s_[k] & 0x80000000u) | (s_[(k + 1) % kN] & 0x7fffffffu);
        s_[k] = s_[(k + 397) % kN] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
      }
      i_ = 0;
    }
    uint32_t y = s_[i_++];
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= y >> 18;
    return y;
  }
  double sample() {
    const uint32_t a = next() >> 5, b = next() >> 6;
    return (a * 67108864.0 + b) / 9007199254740992.0;
  }

 private:
  static constexpr int kN = 624;
  uint32_t s_[kN];
  int i_ = kN;
};

// Uploads the tables of the random tracer once per device, outside a
// stream capture (a capture that meets them missing gets CMM_ERR_ARG).
int ensure_random_tables(cudaStream_t s) {
  static std::mutex mu;
  static bool done[64] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cmm_tracer_eval");
  if (dev < 0 || dev >= 64) {
    set_last_error("cmm_tracer_eval: device ordinal out of range");
    return CMM_ERR_ARG;
  }
  std::lock_guard<std::mutex> lock(mu);
  if (done[dev]) return CMM_OK;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if ((e = cudaStreamIsCapturing(s, &cs)) != cudaSuccess) return cuda_fail(e, "cmm_tracer_eval");
  if (cs != cudaStreamCaptureStatusNone) {
    set_last_error("cmm_tracer_eval: call the random tracer once outside a stream capture first");
    return CMM_ERR_ARG;
  }
  // coefficient lm = l(l-1) + l + m, the order of the reference's double loop
  Mt19937 rng(42);
  double c[kRandW * kRandW];
  for (double& v : c) v = -1.0 + 2.0 * rng.sample();
  double A[kRandW * kRandW] = {}, ab[2 * kRandW * kRandW] = {}, fm[kRandW] = {};
  for (int l = 1; l <= kRandL; ++l) {
    const int base = l * (l - 1) + l;
    A[l] = c[base];                                        // m = 0
    for (int m = 1; m < l; ++m)
      A[m * kRandW + l] = c[base + m] + ((m & 1) ? -c[base - m] : c[base - m]);
    A[l * kRandW + l] = (l & 1) ? -c[base - l] : c[base - l];  // m = l: only Y_l^-l
  }
  for (int m = 0; m <= kRandL; ++m) {
    if (m > 0) fm[m] = std::sqrt((2.0 * m + 1) / (2.0 * m));
    double a_prev = 0.0;
    for (int l = m + 1; l <= kRandL; ++l) {
      const double a = std::sqrt((4.0 * l * l - 1) / ((double)l * l - (double)m * m));
      ab[2 * (m * kRandW + l)] = a;
      ab[2 * (m * kRandW + l) + 1] = a_prev > 0.0 ? 1.0 / a_prev : 0.0;
      a_prev = a;
    }
  }
  if ((e = cudaMemcpyToSymbol(c_rand_A, A, sizeof(A))) != cudaSuccess ||
      (e = cudaMemcpyToSymbol(c_rand_ab, ab, sizeof(ab))) != cudaSuccess ||
      (e = cudaMemcpyToSymbol(c_rand_fm, fm, sizeof(fm))) != cudaSuccess)
    return cuda_fail(e, "cmm_tracer_eval: random tracer tables");
  done[dev] = true;
  return CMM_OK;
}

}  // namespace

int launch_tracer(const MeshView& m, int kind, double t, const double* X, int64_t n, double* out,
                  cudaStream_t s) {
  if (kind < CMM_TRACER_COSINE_BELL || kind > CMM_TRACER_RANDOM_SH) {
    set_last_error("cmm_tracer_eval: unknown tracer");
    return CMM_ERR_ARG;
  }
  TracerSpec ts{};
  ts.kind = kind;
  ts.t = t;
  double A[9], B[9], Bt[9];
  rot_x(kPi / 2, A);
  rot_z(0.0, B);
  transpose3(B, Bt);
  matmul3(A, Bt, ts.rot);
  if (n == 0) return CMM_OK;
  if (kind == CMM_TRACER_RANDOM_SH) {
    const int rc = ensure_random_tables(s);
    if (rc) return rc;
  }
  tracer_kernel<<<grid_for(n, kBlock), kBlock, 0, s>>>(m, ts, X, n, out);
  return check_launch("tracer_kernel");
}

}  // namespace cmm
