// Velocity interpolant on the MWSS lat-lon mesh, backward integrators and
// the CMM map update (sm_103a).
//
// Location on the lat-lon mesh restates structure_spherical_triangulation
// .inds / .containing_simplex_and_bcc_structured
// (cmm_s2/core/mesh_functions.py:196-282): ring and sector from the angles
// with numpy's floor-division semantics, the reference's near-row
// corrections (theta_c <= 0.03 / > 0.85, great-circle side tests with
// heaviside(0) = 0) and the diagonal side test.  CUDA's atan2/sin/cos are
// not numpy's, so a query exactly on a ring, meridian or diagonal (a
// triangle edge or vertex) may resolve to the other triangle that also
// contains it.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "cmm_internal.h"
#include "device_common.cuh"
#include "geom.h"
#include "integrators.cuh"

namespace cmm {

using namespace dev;

namespace {

constexpr int kBlock = 128;
constexpr int kMaxBlock = 256;   // bound of the tunable advect kernel

// Velocity at q: the Powell-Sabin patch of each time level, combined with
// the stage's Lagrange weights w (spline_interp_velocity.__call__,
// cmm_s2/core/spherical_spline.py:570-615).
struct W3 {
  double a, b, c;
};

__device__ __forceinline__ W3 stage(const TimeWeights& tw, int s) {
  return W3{tw.w[s][0], tw.w[s][1], tw.w[s][2]};
}

__device__ __forceinline__ void velocity_at(const MeshView& m, const VelPtrs& vc, int nvs,
                                            const W3 w, double x, double y, double z,
                                            double* V) {
  const int t = latlon_locate(m, x, y, z);
  V[0] = V[1] = V[2] = 0.0;
  if (m.rec32) {  // FP32 records: barycentrics, patches and time combination in FP32
    const float* Lf = m.tri_loc_f + (int64_t)t * kLocStride;
    float Lr[13];
#pragma unroll
    for (int k = 0; k < 13; ++k) Lr[k] = __ldg(Lf + k);
    const BccF b = bcc_rel_f(m, t, Lr, x, y, z);
    const Split sp = split_of_f(b);
    float gg[3];
    gamma_of_f(Lr, b, sp, gg);
    const float gV = gg[0], gE = gg[1], gC = gg[2];
    float Vf[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int l = 0; l < 3; ++l) {
      if (l >= nvs) break;
      const float wl = to_f32_trunc(l == 0 ? w.a : (l == 1 ? w.b : w.c));
      OrdsF<3> o;
      load_ords_f<3>((const float*)vc.p[l] + (int64_t)t * kCoeffStride3, sp, o);
      float P[3];
      sbb_f<3>(o, gV, gE, gC, P);
      Vf[0] += wl * P[0];
      Vf[1] += wl * P[1];
      Vf[2] += wl * P[2];
    }
    V[0] = Vf[0];
    V[1] = Vf[1];
    V[2] = Vf[2];
    return;
  }
  double Lr[13];
  load_loc(m, t, Lr);
  const Bcc b = bcc_of(Lr, x, y, z);
  const Split sp = split_of(b);
  const Gam g = gamma_of(Lr, b, sp);
#pragma unroll
  for (int l = 0; l < 3; ++l) {
    if (l >= nvs) break;
    const double wl = l == 0 ? w.a : (l == 1 ? w.b : w.c);
    Ords<3> o;
    load_ords<3>(vc.p[l] + (int64_t)t * kCoeffStride3, sp, o);
    double P[3];
    sbb<3>(o, g, P);
    V[0] += wl * P[0];
    V[1] += wl * P[1];
    V[2] += wl * P[2];
  }
}

// The spline velocity as the integrators' velocity source: stage s uses
// the Lagrange weights of the scheme's s-th evaluation time.
struct SplineVel {
  const MeshView& m;
  const VelPtrs& vc;
  int nvs;
  const TimeWeights& tw;
  __device__ __forceinline__ void operator()(int s, double x, double y, double z, double* V) const {
    velocity_at(m, vc, nvs, stage(tw, s), x, y, z, V);
  }
};

__device__ __forceinline__ void integrate_point(const MeshView& m, const VelPtrs& vc, int nvs,
                                                const TimeWeights& tw, int scheme, double dt,
                                                double* x) {
  integrate_back(SplineVel{m, vc, nvs, tw}, scheme, dt, x);
}

__global__ void __launch_bounds__(kBlock) latlon_locate_kernel(MeshView m, const double* __restrict__ q,
                                                               int64_t n, int32_t* __restrict__ tri,
                                                               double* __restrict__ bcc) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double x = q[3 * i], y = q[3 * i + 1], z = q[3 * i + 2];
    if (!finite3(x, y, z)) {
      flag(m, CMM_FLAG_NONFINITE);
      tri[i] = -1;
      if (bcc) bcc[3 * i] = bcc[3 * i + 1] = bcc[3 * i + 2] = nan("");
      continue;
    }
    const int t = latlon_locate(m, x, y, z);
    tri[i] = t;
    if (bcc) {
      const Bcc b = bcc_of(m.tri_loc + (int64_t)t * kLocStride, x, y, z);
      bcc[3 * i] = b.b0;
      bcc[3 * i + 1] = b.b1;
      bcc[3 * i + 2] = b.b2;
    }
  }
}

// x, out: (3,n) component-major, as the reference's (3,N) arrays.
__global__ void __launch_bounds__(kBlock) velocity_kernel(MeshView m, VelPtrs vc, int nvs,
                                                          TimeWeights tw, const double* __restrict__ x,
                                                          int64_t n, double* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double px = x[i], py = x[n + i], pz = x[2 * n + i];
    double V[3] = {nan(""), nan(""), nan("")};
    if (finite3(px, py, pz))
      velocity_at(m, vc, nvs, stage(tw, 0), px, py, pz, V);
    else
      flag(m, CMM_FLAG_NONFINITE);
    out[i] = V[0];
    out[n + i] = V[1];
    out[2 * n + i] = V[2];
  }
}

__global__ void __launch_bounds__(kBlock) integrate_kernel(MeshView m, VelPtrs vc, int nvs,
                                                           TimeWeights tw, int scheme, double dt,
                                                           const double* __restrict__ x, int64_t n,
                                                           double* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double p[3] = {x[i], x[n + i], x[2 * n + i]};
    if (finite3(p[0], p[1], p[2])) {
      integrate_point(m, vc, nvs, tw, scheme, dt, p);
      if (!finite3(p[0], p[1], p[2])) flag(m, CMM_FLAG_NONFINITE);
    } else {
      flag(m, CMM_FLAG_NONFINITE);
    }
    out[i] = p[0];
    out[n + i] = p[1];
    out[2 * n + i] = p[2];
  }
}

// Foot points of the mesh vertices and of their stencil points
// (advect, cmm_s2/core/evolution_functions.py:117-133).  Point i < nv is
// vertex i, point nv + k*nv + v is stencil point k of vertex v.  work:
// yn (3,nv) followed by the stencil foot points (3,4,nv).  Register cap
// for 3 blocks of 256 (6 of 128) per SM: 80 registers and a few spills
// beat 120 registers at 16 warps by 4-6 %.
__global__ void __launch_bounds__(kMaxBlock, 3) advect_points_kernel(MeshView mesh, MeshView vm, VelPtrs vc,
                                                               int nvs, TimeWeights tw, int scheme,
                                                               double dt,
                                                               const double* __restrict__ s_pts,
                                                               double* __restrict__ work,
                                                               const BveState* __restrict__ st) {
  if (st) {
    vc = VelPtrs{{st->vel[0], st->vel[1], st->vel[2]}};
    tw = st->tw;
  }
  const int64_t nv = mesh.nv, n = 5 * nv;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double p[3];
    if (i < nv) {
      p[0] = mesh.verts[4 * i];
      p[1] = mesh.verts[4 * i + 1];
      p[2] = mesh.verts[4 * i + 2];
    } else {
      const int64_t j = i - nv;  // k*nv + v within the (3, 4nv) stencil array
      p[0] = s_pts[j];
      p[1] = s_pts[4 * nv + j];
      p[2] = s_pts[8 * nv + j];
    }
    integrate_point(vm, vc, nvs, tw, scheme, dt, p);
    if (!finite3(p[0], p[1], p[2])) flag(vm, CMM_FLAG_NONFINITE);
    if (i < nv) {
      work[i] = p[0];
      work[nv + i] = p[1];
      work[2 * nv + i] = p[2];
    } else {
      const int64_t j = i - nv;
      double* sn = work + 3 * nv;
      sn[j] = p[0];
      sn[4 * nv + j] = p[1];
      sn[8 * nv + j] = p[2];
    }
  }
}

// New jets from the stencil images (spline_proj_sphere,
// cmm_s2/core/evolution_functions.py:90-113); with a previous map, the
// images are the previous map evaluated at the stencil foot points in the
// sub-triangle of the vertex foot point, un-normalised (stencil_eval,
// cmm_s2/core/spherical_spline.py:268-298).
__global__ void __launch_bounds__(kBlock) project_jets_kernel(MeshView m, const double* __restrict__ prev,
                                                              const double* __restrict__ yn,
                                                              const double* __restrict__ sn,
                                                              const double* __restrict__ tan,
                                                              double eps, double* __restrict__ jets,
                                                              const BveState* __restrict__ st) {
  const int64_t nv = m.nv;
  const int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (v >= nv) return;
  if (st && st->identity) prev = nullptr;
  double S[4][3];
#pragma unroll
  for (int k = 0; k < 4; ++k)
#pragma unroll
    for (int c = 0; c < 3; ++c) S[k][c] = sn[(c * 4 + k) * nv + v];
  if (prev) {
    const double x = yn[v], y = yn[nv + v], z = yn[2 * nv + v];
    if (!finite3(x, y, z)) {
      flag(m, CMM_FLAG_NONFINITE);
      for (int k = 0; k < 12; ++k) jets[k * nv + v] = nan("");
      return;
    }
    const int t = locate_row(m, x, y, z);
    double Lr[13];
    load_loc(m, t, Lr);
    const Split sp = split_of(bcc_of(Lr, x, y, z));
    Ords<3> o;
    load_ords<3>(prev + (int64_t)t * kCoeffStride3, sp, o);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const Gam g = gamma_of(Lr, bcc_of(Lr, S[k][0], S[k][1], S[k][2]), sp);
      double P[3];
      sbb<3>(o, g, P);
      S[k][0] = P[0];
      S[k][1] = P[1];
      S[k][2] = P[2];
    }
  }
  double mv[3], d1[3], d2[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    mv[c] = (S[0][c] + S[1][c] + S[2][c] + S[3][c]) / 4;
    d1[c] = (S[1][c] - S[0][c] + S[3][c] - S[2][c]) / (4 * eps);
    d2[c] = (S[2][c] - S[0][c] + S[3][c] - S[1][c]) / (4 * eps);
  }
  const double nm = sqrt(mv[0] * mv[0] + mv[1] * mv[1] + mv[2] * mv[2]);
  const double* a1 = tan + 3 * v;
  const double* a2 = tan + 3 * (nv + v);
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    jets[(c * 4 + 0) * nv + v] = mv[c] / nm;
#pragma unroll
    for (int k = 0; k < 3; ++k) jets[(c * 4 + 1 + k) * nv + v] = d1[k] * a1[c] + d2[k] * a2[c];
  }
  if (!finite3(mv[0], mv[1], mv[2])) flag(m, CMM_FLAG_NONFINITE);
}

int check_launch(const char* what) {
  note_launch();
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? CMM_OK : cuda_fail(e, what);
}

}  // namespace

int launch_latlon_locate(const MeshView& vm, const double* q, int64_t n, int32_t* tri, double* bcc,
                         cudaStream_t s) {
  if (n == 0) return CMM_OK;
  latlon_locate_kernel<<<grid_for(n, kBlock), kBlock, 0, s>>>(vm, q, n, tri, bcc);
  return check_launch("latlon_locate_kernel");
}

int launch_velocity_eval(const MeshView& vm, VelPtrs vc, int nvs, const TimeWeights& tw,
                         const double* x, int64_t n, double* out, cudaStream_t s) {
  if (n == 0) return CMM_OK;
  velocity_kernel<<<grid_for(n, kBlock), kBlock, 0, s>>>(vm, vc, nvs, tw, x, n, out);
  return check_launch("velocity_kernel");
}

int launch_integrate(const MeshView& vm, VelPtrs vc, int nvs, const TimeWeights& tw, int scheme,
                     double dt, const double* x, int64_t n, double* out, cudaStream_t s) {
  if (n == 0) return CMM_OK;
  integrate_kernel<<<grid_for(n, kBlock), kBlock, 0, s>>>(vm, vc, nvs, tw, scheme, dt, x, n, out);
  return check_launch("integrate_kernel");
}

int launch_advect_points(const MeshView& mesh, const MeshView& vm, VelPtrs vc, int nvs,
                         const TimeWeights& tw, int scheme, double dt, const double* s_pts,
                         double* work, cudaStream_t s, const BveState* st) {
  const int64_t n = 5LL * mesh.nv;
  const int b = block_for(mesh, kTuneAdvect, kBlock, n);
  advect_points_kernel<<<grid_for(n, b), b, 0, s>>>(mesh, vm, vc, nvs, tw, scheme, dt,
                                                               s_pts, work, st);
  return check_launch("advect_points_kernel");
}

// ---------------------------------------------- allocation-free map update
// Foot-point scratch of advect_project_noalloc: a fixed array in device
// memory that exists on every GPU this library is loaded on, for meshes of
// up to kNoAllocMaxVerts vertices (icosahedral level 5).  Host code must not
// use the name g_advect_scratch as a pointer; the device address of each
// GPU's copy is looked up once per device with cudaGetSymbolAddress.
static __device__ __align__(256) double g_advect_scratch[15 * kNoAllocMaxVerts];

namespace {
constexpr int kMaxDevices = 64;
double* g_scratch_addr[kMaxDevices] = {};
std::mutex g_scratch_mu;
}  // namespace

static int noalloc_scratch(double** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) {
    set_last_error("advect_project_noalloc: device ordinal out of range");
    return CMM_ERR_UNSUPPORTED;
  }
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_advect_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_advect_scratch)");
    g_scratch_addr[dev] = (double*)p;
  }
  *out = g_scratch_addr[dev];
  return CMM_OK;
}

int advect_project_noalloc(const MeshView& mesh, const MeshView& vm, VelPtrs vc, int nvs,
                           const TimeWeights& tw, int scheme, double dt, const double* s_pts,
                           const double* tan, const double* prev_coeffs, double eps,
                           double* jets, cudaStream_t s) {
  if (mesh.nv > kNoAllocMaxVerts) {
    set_last_error("cmm_advect_project_noalloc: mesh has more than " +
                   std::to_string(kNoAllocMaxVerts) +
                   " vertices (icosahedral level 5); use cmm_advect_project with a workspace");
    return CMM_ERR_ARG;
  }
  double* work = nullptr;
  int rc = noalloc_scratch(&work);
  if (rc) return rc;
  // every scratch entry is written by advect_points_kernel before
  // project_jets_kernel reads it, so nothing needs clearing
  if ((rc = launch_advect_points(mesh, vm, vc, nvs, tw, scheme, dt, s_pts, work, s))) return rc;
  return launch_project_jets(mesh, prev_coeffs, work, work + 3 * (int64_t)mesh.nv, tan, eps, jets, s);
}

int launch_project_jets(const MeshView& mesh, const double* prev_coeffs, const double* yn,
                        const double* sn, const double* tan, double eps, double* jets,
                        cudaStream_t s, const BveState* st) {
  const int64_t nv = mesh.nv;
  const int b = small_block(nv, kBlock);
  project_jets_kernel<<<(int)((nv + b - 1) / b), b, 0, s>>>(mesh, prev_coeffs, yn, sn, tan, eps, jets, st);
  return check_launch("project_jets_kernel");
}

}  // namespace cmm
