// Point location, Powell-Sabin assembly, map evaluation and composition
// kernels for the icosahedral mesh (sm_103a).
//
// Location: a query descends the icosahedral refinement hierarchy.  At each
// node three great-circle tests (the planes through the edge midpoints)
// choose one of the four children.  Tests run in FP32 against unit normals
// and are redone in FP64 only when |n.q| < kFilter, inside which the FP32
// sign is not guaranteed (|q| = |n| = 1: the FP32 dot is within ~6e-7 of
// the exact dot of the FP64 inputs).  The FP64 decision equals the
// reference's Qhull choice except for queries within rounding distance of
// an edge, where either neighbour contains the query.
//
// Evaluation: with bcc = Minv q (precomputed inverse vertex matrix per
// triangle) the Powell-Sabin sub-triangle is picked by argmin/argmax of the
// bcc with numpy's first-index tie rule (cmm_s2/core/spherical_spline.py:
// 691-697); the sub-triangle barycentrics follow in closed form from the
// triangle's, since its corners are v_hi, (v_hi+v_mid)/|v_hi+v_mid| and
// (v1+v2+v3)/|v1+v2+v3|:
//     gV = b_hi - b_mid,  gE = |v_hi+v_mid| (b_mid - b_lo),  gC = |v1+v2+v3| b_lo
// which is the same linear map the reference obtains from four 3x3
// determinants (new_vpoints + bary_coords, :668-689).
#include <cuda_runtime.h>

#include <algorithm>

#include "cmm_internal.h"
#include "dd.cuh"
#include "device_common.cuh"
#include "ff.cuh"

namespace cmm {

using namespace dev;

namespace {

constexpr int kBlock = 256;
// The composition normalises the point every kNormEvery submaps (a power
// of two); queries whose FP32 squared norm is outside [1/4, 4] are
// normalised first, so the unnormalised chain stays far from overflow.
constexpr int kNormEvery = 8;
// default register budgets of the compositions, as resident 256-thread
// blocks per SM (measured at level 7, 2^24 queries, 8 submaps, map forms,
// cell order, normalising every fourth submap: Jacobians 12.8 / 13.6 /
// 13.2 ms at 4 / 3 / 2 blocks; points only 7.5 ms at 4 or 6 blocks, and
// 10.2 against 13.5 ms in caller order); the autotuner may set others
constexpr int kComposeJacBlocks = 4;
// with the low floats of the forms' split loaded (fewer live values):
// 10.83 / 11.02 / 11.59 ms at 3 / 4 / 2 blocks, same workload; normalising
// every eighth submap, 10.56 / 10.72 / 11.93 ms
constexpr int kComposeJacBlocksFF = 3;
constexpr int kComposeBlocks = 4;

// Submap lists: by value in the kernel parameters (host calls), or a
// device table whose length comes from a device-driven step's state.
// Each submap has its coefficient record and, optionally, its map-form
// record (form(s) != NULL: evaluated as quadratic forms).
// A submap with a form record may also have the low floats of its
// float-float split (the Jacobian pushes then load them instead of
// extracting them from the doubles on the integer pipe).
struct SubmapPtrs {
  const double* p[CMM_MAX_SUBMAPS];
  const double* f[CMM_MAX_SUBMAPS];
  const float* g[CMM_MAX_SUBMAPS];
  int S;
  __device__ __forceinline__ int count() const { return S; }
  __device__ __forceinline__ const double* at(int s, int) const { return p[s]; }
  __device__ __forceinline__ const double* form(int s, int) const { return f[s]; }
  __device__ __forceinline__ const float* form_ff(int s, int) const { return g[s]; }
};
struct DevSubmaps {
  const double* const* tab;
  const double* const* ftab;   // forms of the stack slots, or NULL
  const BveState* st;
  const double* last;
  __device__ __forceinline__ int count() const { return st->nc + 1; }
  __device__ __forceinline__ const double* at(int s, int S) const { return s < S - 1 ? tab[s] : last; }
  __device__ __forceinline__ const double* form(int s, int S) const {
    return ftab && s < S - 1 ? ftab[s] : nullptr;
  }
  __device__ __forceinline__ const float* form_ff(int, int) const { return nullptr; }
};

// Orthonormal tangent basis (t1, t2) at the unit point p, in float-float
// from the FP64 point (the Jacobian's tangent pushes run in float-float on
// the FP32 pipe).
__device__ __forceinline__ void tangent_basis_ff(const double* p, ff* t1, ff* t2) {
  const ff p0 = ff_of(p[0]), p1 = ff_of(p[1]), p2 = ff_of(p[2]);
  const bool polar = !(fabsf(p2.h) < 0.9f);
  // t1 = e x p normalised, e = z (or x near the poles): (p1, -p0, 0) or (0, p2, -p1)
  const ff a = polar ? p2 : p1, b = polar ? ff_neg(p1) : ff_neg(p0);
  const ff r = ff_rsqrt(ff_dot2(a, a, b, b));
  const ff ua = ff_mul(a, r), ub = ff_mul(b, r);
  const ff z{0.f, 0.f};
  t1[0] = polar ? z : ua;
  t1[1] = polar ? ua : ub;
  t1[2] = polar ? ub : z;
  // t2 = p x t1
  t2[0] = ff_sub(ff_mul(p1, t1[2]), ff_mul(p2, t1[1]));
  t2[1] = ff_sub(ff_mul(p2, t1[0]), ff_mul(p0, t1[2]));
  t2[2] = ff_sub(ff_mul(p0, t1[1]), ff_mul(p1, t1[0]));
}

__device__ __forceinline__ ff pick_ff(const ff* b, int i) { return i == 0 ? b[0] : (i == 1 ? b[1] : b[2]); }

// Twelve float-float values of one thread in shared memory, value-major
// (value k at s[2k * stride], s[(2k + 1) * stride]: conflict-free): the two
// tangent pushes (0..5) and their barycentric directions (6..11).
struct Pushes {
  float* s;
  int stride;
  __device__ __forceinline__ ff get(int k) const { return ff{s[2 * k * stride], s[(2 * k + 1) * stride]}; }
  __device__ __forceinline__ void set(int k, ff v) {
    s[2 * k * stride] = v.h;
    s[(2 * k + 1) * stride] = v.l;
  }
};

// 2^m as a double, from its bit pattern (0 <= m <= kNormEvery here)
__device__ __forceinline__ double pow2(int m) { return __longlong_as_double((long long)(1023 + m) << 52); }

__global__ void __launch_bounds__(kBlock) locate_kernel(MeshView m, const double* __restrict__ q,
                                                        int64_t n, int32_t* __restrict__ tri,
                                                        double* __restrict__ bcc) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double x = q[3 * i], y = q[3 * i + 1], z = q[3 * i + 2];
    if (!finite3(x, y, z)) {
      flag(m, CMM_FLAG_NONFINITE);
      tri[i] = -1;
      if (bcc) bcc[3 * i] = bcc[3 * i + 1] = bcc[3 * i + 2] = nan("");
      continue;
    }
    int t = locate_row(m, x, y, z);
    tri[i] = t;
    if (bcc) {
      Bcc b = bcc_of(m.tri_loc + (int64_t)t * kLocStride, x, y, z);
      bcc[3 * i] = b.b0;
      bcc[3 * i + 1] = b.b1;
      bcc[3 * i + 2] = b.b2;
      if (fmin(b.b0, fmin(b.b1, b.b2)) < -1e-10) flag(m, CMM_FLAG_LOCATE);
    }
  }
}

// One triangle per thread: the 19 ordinates of each component from the
// jets of its three vertices (assemble_coefficients,
// cmm_s2/core/spherical_spline.py:300-337) using the per-triangle factors
// (factor-major, coalesced loads).  The block's records are staged in
// shared memory (rows padded to stride+1 doubles against bank conflicts)
// and written out as one contiguous, coalesced range, record padding
// included (zeros).
constexpr int kAsmTri = 64;   // triangles (threads) per block

template <int NC>
__global__ void __launch_bounds__(kAsmTri) assemble_kernel(MeshView m, const double* __restrict__ jets,
                                                           double* __restrict__ coeffs,
                                                           const BveState* __restrict__ st) {
  if (st) coeffs = st->vel[0];
  constexpr int kStride = NC == 3 ? kCoeffStride3 : kCoeffStride1;
  constexpr int kRow = kStride + 1;
  __shared__ double rec[kAsmTri * kRow];
  const int t0 = blockIdx.x * kAsmTri;
  const int nblk = min(kAsmTri, m.nt - t0);
  const int tl = threadIdx.x, t = t0 + tl;
  double* out = rec + tl * kRow;
  if (tl < nblk) {
    const int nv = m.nv, nt = m.nt;
    const int4 tv = m.tri_v[t];
    const int vid[3] = {tv.x, tv.y, tv.z};
    const double* A = m.tri_asm + t;   // factor j at A[j * nt]
    const int corner[9] = {0, 0, 0, 1, 1, 1, 2, 2, 2};
#pragma unroll
    for (int k = 0; k < NC; ++k) {
      double f[3], c[19];
#pragma unroll
      for (int v = 0; v < 3; ++v) f[v] = __ldg(jets + (int64_t)(k * 4) * nv + vid[v]);
      c[0] = f[0];
      c[1] = f[1];
      c[2] = f[2];
#pragma unroll
      for (int o = 0; o < 9; ++o) {
        const int v = vid[corner[o]];
        double gx, gy, gz;
        if (NC == 3) {  // d_j f_k = jets[j][1+k]
          gx = __ldg(jets + (int64_t)(0 * 4 + 1 + k) * nv + v);
          gy = __ldg(jets + (int64_t)(1 * 4 + 1 + k) * nv + v);
          gz = __ldg(jets + (int64_t)(2 * 4 + 1 + k) * nv + v);
        } else {  // scalar: d_j f = jets[1+j]
          gx = __ldg(jets + (int64_t)1 * nv + v);
          gy = __ldg(jets + (int64_t)2 * nv + v);
          gz = __ldg(jets + (int64_t)3 * nv + v);
        }
        const double a0 = __ldg(A + (int64_t)(4 * o) * nt), a1 = __ldg(A + (int64_t)(4 * o + 1) * nt),
                     a2 = __ldg(A + (int64_t)(4 * o + 2) * nt), a3 = __ldg(A + (int64_t)(4 * o + 3) * nt);
        c[3 + o] = a0 * gx + a1 * gy + a2 * gz - a3 * f[corner[o]];
      }
      double e[9];
#pragma unroll
      for (int j = 0; j < 9; ++j) e[j] = __ldg(A + (int64_t)(36 + j) * nt);
      c[12] = e[0] * c[3] + e[1] * c[8];
      c[13] = e[2] * c[6] + e[3] * c[11];
      c[14] = e[5] * c[9] + e[4] * c[5];
      c[15] = e[0] * c[4] + e[1] * c[7];
      c[16] = e[2] * c[7] + e[3] * c[10];
      c[17] = e[4] * c[4] + e[5] * c[10];
      c[18] = e[6] * c[4] + e[7] * c[7] + e[8] * c[10];
#pragma unroll
      for (int o = 0; o < 19; ++o) out[NC * o + k] = c[o];
    }
#pragma unroll
    for (int j = 19 * NC; j < kStride; ++j) out[j] = 0.0;
  }
  __syncthreads();
  double* dst = coeffs + (int64_t)t0 * kStride;
  for (int i = tl; i < nblk * kStride; i += kAsmTri) dst[i] = rec[(i / kStride) * kRow + i % kStride];
}

// FP32 velocity records (velmesh with rec32, ncomp = 3): the same
// ordinates from FP32 jets and the FP32 factor table, in FP32.  J: the
// jets' storage type (double jets are rounded to float here; float jets
// are the split form's FP32 jets, the same values without conversions).
template <typename J>
__global__ void __launch_bounds__(kAsmTri) assemble_f32_kernel(MeshView m, const J* __restrict__ jets,
                                                               float* __restrict__ coeffs,
                                                               const BveState* __restrict__ st) {
  if (st) coeffs = (float*)st->vel[0];
  constexpr int kStride = kCoeffStride3;
  constexpr int kRow = kStride + 1;
  __shared__ float rec[kAsmTri * kRow];
  const int t0 = blockIdx.x * kAsmTri;
  const int nblk = min(kAsmTri, m.nt - t0);
  const int tl = threadIdx.x, t = t0 + tl;
  float* out = rec + tl * kRow;
  if (tl < nblk) {
    const int nv = m.nv, nt = m.nt;
    const int4 tv = m.tri_v[t];
    const int vid[3] = {tv.x, tv.y, tv.z};
    const float* A = m.tri_asm_f + t;
    const int corner[9] = {0, 0, 0, 1, 1, 1, 2, 2, 2};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      float f[3], c[19];
#pragma unroll
      for (int v = 0; v < 3; ++v) f[v] = (float)__ldg(jets + (int64_t)(k * 4) * nv + vid[v]);
      c[0] = f[0];
      c[1] = f[1];
      c[2] = f[2];
#pragma unroll
      for (int o = 0; o < 9; ++o) {
        const int v = vid[corner[o]];
        const float gx = (float)__ldg(jets + (int64_t)(0 * 4 + 1 + k) * nv + v);
        const float gy = (float)__ldg(jets + (int64_t)(1 * 4 + 1 + k) * nv + v);
        const float gz = (float)__ldg(jets + (int64_t)(2 * 4 + 1 + k) * nv + v);
        c[3 + o] = __ldg(A + (int64_t)(4 * o) * nt) * gx + __ldg(A + (int64_t)(4 * o + 1) * nt) * gy +
                   __ldg(A + (int64_t)(4 * o + 2) * nt) * gz - __ldg(A + (int64_t)(4 * o + 3) * nt) * f[corner[o]];
      }
      float e[9];
#pragma unroll
      for (int j = 0; j < 9; ++j) e[j] = __ldg(A + (int64_t)(36 + j) * nt);
      c[12] = e[0] * c[3] + e[1] * c[8];
      c[13] = e[2] * c[6] + e[3] * c[11];
      c[14] = e[5] * c[9] + e[4] * c[5];
      c[15] = e[0] * c[4] + e[1] * c[7];
      c[16] = e[2] * c[7] + e[3] * c[10];
      c[17] = e[4] * c[4] + e[5] * c[10];
      c[18] = e[6] * c[4] + e[7] * c[7] + e[8] * c[10];
#pragma unroll
      for (int o = 0; o < 19; ++o) out[3 * o + k] = c[o];
    }
#pragma unroll
    for (int j = 57; j < kStride; ++j) out[j] = 0.f;
  }
  __syncthreads();
  float* dst = coeffs + (int64_t)t0 * kStride;
  for (int i = tl; i < nblk * kStride; i += kAsmTri) dst[i] = rec[(i / kStride) * kRow + i % kStride];
}

// Map forms: one thread per (triangle, sub-triangle).  The sub-triangle
// barycentrics are gamma = T p with rows T_V = R_hi - R_mid,
// T_E = |v_hi + v_mid| (R_mid - R_lo), T_C = |v1 + v2 + v3| R_lo (R the
// inverse vertex rows of the location record), so the patch
// P_c = gamma^T M_c gamma (M_c the symmetric matrix of the sub-triangle's
// six ordinates) is the homogeneous quadratic form p^T Q_c p with
// Q_c = T^T M_c T.  Q is O(1) while T is O(1/h), so its entries cancel
// terms ~1/h^2 times larger: T, M_c T and Q_c are formed in double-double
// and rounded once.  The result is the exact quadratic form of the patch
// the record's rows R define, and p^T Q p then evaluates in FP64 without
// cancellation (~2e-16 against the Bernstein sum's ~1e-14 from R p).
__device__ __forceinline__ void assemble_form(const MeshView& m, const double* __restrict__ coeffs,
                                              double* __restrict__ forms, int64_t idx) {
  const int t = (int)(idx / 6), sub = (int)(idx % 6);
  const int lo = kSubLo[sub], hi = kSubHi[sub], mid = 3 - lo - hi;
  const double* L = m.tri_loc + (int64_t)t * kLocStride;
  const double ne = edge_norm(L, hi, mid), n4 = __ldg(L + 9);
  dd T[3][3];   // rows V, E, C
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    const double rh = __ldg(L + 3 * hi + j), rm = __ldg(L + 3 * mid + j), rl = __ldg(L + 3 * lo + j);
    T[0][j] = dd_two_sum(rh, -rm);
    T[1][j] = dd_mul_d(dd_two_sum(rm, -rl), ne);
    T[2][j] = dd_two_prod(n4, rl);
  }
  const int* id = kSplitOrd[lo][hi];   // V^2, E^2, C^2, VE, EC, VC
  const double* rec = coeffs + (int64_t)t * kCoeffStride3;
  double* out = forms + (int64_t)t * kFormStride + 18 * sub;
  // M_c = [[V2, VE, VC], [VE, E2, EC], [VC, EC, C2]] of each component
  double M[3][6];   // per component: the pairs (VV, EE, CC, VE, EC, VC)
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int k = 0; k < 6; ++k) M[c][k] = __ldg(rec + 3 * id[k] + c);
  // Q_c[i][j] = sum over role pairs a <= b of M_c,ab P_ab[i][j] with
  // P_aa = T_a,i T_a,j and P_ab = T_a,i T_b,j + T_b,i T_a,j (a < b):
  // symmetric in (i, j) by construction, so the stored 2 Q_ij is exact
  const int pa[6] = {0, 1, 2, 0, 1, 0}, pb[6] = {0, 1, 2, 1, 2, 2};   // VV, EE, CC, VE, EC, VC
  const int ei[6] = {0, 1, 2, 0, 0, 1}, ej[6] = {0, 1, 2, 1, 2, 2};   // xx, yy, zz, xy, xz, yz
#pragma unroll
  for (int e = 0; e < 6; ++e) {
    const int i = ei[e], j = ej[e];
    dd P[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      const int a = pa[k], b = pb[k];
      P[k] = a == b ? dd_mul(T[a][i], T[a][j]) : dd_add_fast(dd_mul(T[a][i], T[b][j]), dd_mul(T[b][i], T[a][j]));
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const double q = dd_dot_d(P, M[c]);
      out[6 * c + e] = i == j ? q : 2.0 * q;
    }
  }
  if (sub == 0)
    for (int k = 108; k < kFormStride; ++k) forms[(int64_t)t * kFormStride + k] = 0.0;
}

__global__ void __launch_bounds__(128) assemble_forms_kernel(MeshView m, const double* __restrict__ coeffs,
                                                             double* __restrict__ forms) {
  const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (idx < 6LL * m.nt) assemble_form(m, coeffs, forms, idx);
}

// The device-driven step's remap: the forms of the stack slot the current
// map has just been copied to (st->count + 1 in the remap schedule), a
// no-op on the other steps.
__global__ void __launch_bounds__(128) remap_forms_kernel(MeshView m, const BveState* __restrict__ st, int n_maps,
                                                          int Nt, const double* const* __restrict__ table,
                                                          double* const* __restrict__ ftable) {
  const int c = st->count + 1;
  const int slot = c == Nt ? (Nt - 1) / n_maps : (c < Nt && c % n_maps == 0 ? c / n_maps - 1 : -1);
  if (slot < 0) return;
  const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (idx < 6LL * m.nt) assemble_form(m, table[slot], ftable[slot], idx);
}

// Low floats of the form records' float-float split: one thread per
// (triangle, sub-triangle, component), the low floats of ff_of of the six
// entries of Q, the cross terms halved (exact), written as three float2
// (padding floats zeroed).
__global__ void __launch_bounds__(128) forms_ff_kernel(int nt, const double* __restrict__ forms,
                                                       float* __restrict__ out) {
  const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (idx >= 18LL * nt) return;
  const int t = (int)(idx / 18), sc = (int)(idx % 18);   // sc = 3 sub + c
  const double* q = forms + (int64_t)t * kFormStride + 6 * sc;
  float2* o = reinterpret_cast<float2*>(out + (int64_t)t * kFormFFStride + 6 * sc);
  o[0] = make_float2(ff_of(q[0]).l, ff_of(q[1]).l);
  o[1] = make_float2(ff_of(q[2]).l, __fmul_rn(0.5f, ff_of(q[3]).l));
  o[2] = make_float2(__fmul_rn(0.5f, ff_of(q[4]).l), __fmul_rn(0.5f, ff_of(q[5]).l));
  if (sc == 0)
    for (int k = 108; k < kFormFFStride; ++k) out[(int64_t)t * kFormFFStride + k] = 0.f;
}

__global__ void to_f32_kernel(const double* __restrict__ a, int64_t n, float* __restrict__ b) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) b[i] = (float)a[i];
}

// perm (nullable): process the queries in this order (grouped by coarse
// cell, cmm_query_order) so that neighbouring threads gather neighbouring
// records; every query's own arithmetic and output slot are unchanged.
// MINB: resident 256-thread blocks per SM the register allocation must
// allow (the register budget; cmm_mesh_set_variant).  FF: every submap
// with a form record also has the low floats of its float-float split.
template <bool JAC, class Src, int MINB, bool FF = false>
__global__ void __launch_bounds__(kBlock, MINB) compose_kernel(MeshView m, Src cp,
                                                         const double* __restrict__ q, int64_t n,
                                                         double* __restrict__ out,
                                                         int32_t* __restrict__ tri,
                                                         int32_t* __restrict__ tri_all,
                                                         double* __restrict__ jac,
                                                         const int32_t* __restrict__ perm) {
  __shared__ float push_smem[JAC ? 24 * kBlock : 1];
  const int S = cp.count();
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n;
       j += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = perm ? (int64_t)__ldg(perm + j) : j;
    if ((uint64_t)i >= (uint64_t)n) {   // a bad permutation entry
      flag(m, CMM_FLAG_INDEX);
      continue;
    }
    double p[3] = {q[3 * i], q[3 * i + 1], q[3 * i + 2]};
    {
      const float f0 = to_f32_trunc(p[0]), f1 = to_f32_trunc(p[1]), f2 = to_f32_trunc(p[2]);
      const float n2 = f0 * f0 + f1 * f1 + f2 * f2;
      if (!(n2 > 0.25f && n2 < 4.f)) {   // also NaN / inf: then the check below flags it
        const double inv = rsqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
        p[0] *= inv;
        p[1] *= inv;
        p[2] *= inv;
      }
    }
    if (!finite3(p[0], p[1], p[2])) {
      flag(m, CMM_FLAG_NONFINITE);
      out[3 * i] = out[3 * i + 1] = out[3 * i + 2] = nan("");
      if (tri) tri[i] = -1;
      if (tri_all)
        for (int s = 0; s < S; ++s) tri_all[(int64_t)s * n + i] = -1;
      if (JAC)
        for (int k = 0; k < 9; ++k) jac[9 * i + k] = nan("");
      continue;
    }
    // Jacobian: two tangent vectors pushed through the chain in
    // float-float on the FP32 pipe (the points, the location predicates,
    // the barycentrics and the patch values stay FP64)
    // The pushes live in shared memory, [value][thread], not in
    // registers: with them the loop exceeds the register budget of four
    // resident blocks and spills to local memory, whose traffic thrashes
    // the L1 that the gathers need.
    Pushes w{push_smem + threadIdx.x, (int)blockDim.x};
    int since = 0;   // submaps pushed since the last normalisation
    if (JAC) {   // pushed from the tangent basis at q
      ff t1[3], t2[3];
      tangent_basis_ff(p, t1, t2);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        w.set(c, t1[c]);
        w.set(3 + c, t2[c]);
      }
    }
    for (int s = S - 1; s >= 0; --s) {
      double P[3];
      const double* fr = cp.form(s, S);
      if (fr) {
        // map-form record: P_c = p^T Q_c p of the sub-triangle's quadratic
        // form (24 FP64 operations for the three components); the half
        // derivative along w is (Q_c p) . w, formed in float-float
        Split sp;
        const int t = locate_split(m, p[0], p[1], p[2], &sp);
        if (s == S - 1 && tri) tri[i] = t;
        if (tri_all) tri_all[(int64_t)s * n + i] = t;
        const double2* qf =
            reinterpret_cast<const double2*>(fr + (int64_t)t * kFormStride + 18 * kSubIndex[sp.lo][sp.hi]);
        const double xx = p[0] * p[0], yy = p[1] * p[1], zz = p[2] * p[2];
        const double xy = p[0] * p[1], xz = p[0] * p[2], yz = p[1] * p[2];
        if (JAC) {
          const ff u0 = ff_of(p[0]), u1 = ff_of(p[1]), u2 = ff_of(p[2]);
          const ff a0 = w.get(0), a1 = w.get(1), a2 = w.get(2), c0 = w.get(3), c1 = w.get(4), c2 = w.get(5);
          const float2* qg =
              FF ? reinterpret_cast<const float2*>(cp.form_ff(s, S) + (int64_t)t * kFormFFStride +
                                                   18 * kSubIndex[sp.lo][sp.hi])
                 : nullptr;
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            const double2 q01 = __ldg(qf + 3 * c), q23 = __ldg(qf + 3 * c + 1), q45 = __ldg(qf + 3 * c + 2);
            P[c] = q01.x * xx + q01.y * yy + q23.x * zz + q23.y * xy + q45.x * xz + q45.y * yz;
            ff Q00, Q11, Q22, Q01, Q02, Q12;
            if (FF) {   // the stored low floats; the high floats from the doubles' bits
              const float2 ga = __ldg(qg + 3 * c), gb = __ldg(qg + 3 * c + 1), gc = __ldg(qg + 3 * c + 2);
              Q00 = ff{ff_hi(q01.x), ga.x};
              Q11 = ff{ff_hi(q01.y), ga.y};
              Q22 = ff{ff_hi(q23.x), gb.x};
              Q01 = ff{__fmul_rn(0.5f, ff_hi(q23.y)), gb.y};
              Q02 = ff{__fmul_rn(0.5f, ff_hi(q45.x)), gc.x};
              Q12 = ff{__fmul_rn(0.5f, ff_hi(q45.y)), gc.y};
            } else {   // the same pairs converted here
              Q00 = ff_of(q01.x);
              Q11 = ff_of(q01.y);
              Q22 = ff_of(q23.x);
              const ff h01 = ff_of(q23.y), h02 = ff_of(q45.x), h12 = ff_of(q45.y);
              Q01 = ff{__fmul_rn(0.5f, h01.h), __fmul_rn(0.5f, h01.l)};
              Q02 = ff{__fmul_rn(0.5f, h02.h), __fmul_rn(0.5f, h02.l)};
              Q12 = ff{__fmul_rn(0.5f, h12.h), __fmul_rn(0.5f, h12.l)};
            }
            const ff g0 = ff_dot3(Q00, u0, Q01, u1, Q02, u2);
            const ff g1 = ff_dot3(Q01, u0, Q11, u1, Q12, u2);
            const ff g2 = ff_dot3(Q02, u0, Q12, u1, Q22, u2);
            w.set(c, ff_dot3(g0, a0, g1, a1, g2, a2));
            w.set(3 + c, ff_dot3(g0, c0, g1, c1, g2, c2));
          }
          ++since;
        } else {
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            const double2 q01 = __ldg(qf + 3 * c), q23 = __ldg(qf + 3 * c + 1), q45 = __ldg(qf + 3 * c + 2);
            P[c] = q01.x * xx + q01.y * yy + q23.x * zz + q23.y * xy + q45.x * xz + q45.y * yz;
          }
        }
      } else {
      const int t = locate_row(m, p[0], p[1], p[2]);
      if (s == S - 1 && tri) tri[i] = t;
      if (tri_all) tri_all[(int64_t)s * n + i] = t;
      double Lr[13];
      load_loc(m, t, Lr);
      const Bcc b = bcc_of(Lr, p[0], p[1], p[2]);
      const Split sp = split_of(b);
      const Gam g = gamma_of(Lr, b, sp);
      const double* rec = cp.at(s, S) + (int64_t)t * kCoeffStride3;
      if (JAC) {
        // The patch is the quadratic form P_c = gamma^T M_c gamma of the
        // symmetric ordinate matrix M_c; its half gradient M_c gamma (FP64)
        // gives the value with three more operations per component and
        // serves the two tangent pushes: half derivatives along the
        // barycentric directions dgamma = T Minv w, formed in float-float
        // from the FP64 location record.
        // the pushes' sub-triangle barycentric directions, ff values 6..11
        // of the thread's shared-memory slots
        {
          ff d1[3], d2[3];
          // the inverse vertex rows re-read (L1) rather than held in
          // registers from the value path
          const double* Lp = m.tri_loc + (int64_t)t * kLocStride;
#pragma unroll
          for (int r = 0; r < 3; ++r) {
            const ff m0 = ff_of(__ldg(Lp + 3 * r)), m1 = ff_of(__ldg(Lp + 3 * r + 1)),
                     m2 = ff_of(__ldg(Lp + 3 * r + 2));
            d1[r] = ff_dot3(m0, w.get(0), m1, w.get(1), m2, w.get(2));
            d2[r] = ff_dot3(m0, w.get(3), m1, w.get(4), m2, w.get(5));
          }
          const ff en = ff_of(edge_norm(Lr, sp.hi, sp.mid)), ec = ff_of(Lr[9]);
          const ff l1 = pick_ff(d1, sp.lo), m1 = pick_ff(d1, sp.mid), h1 = pick_ff(d1, sp.hi);
          const ff l2 = pick_ff(d2, sp.lo), m2 = pick_ff(d2, sp.mid), h2 = pick_ff(d2, sp.hi);
          w.set(6, ff_sub(h1, m1));
          w.set(7, ff_mul(en, ff_sub(m1, l1)));
          w.set(8, ff_mul(ec, l1));
          w.set(9, ff_sub(h2, m2));
          w.set(10, ff_mul(en, ff_sub(m2, l2)));
          w.set(11, ff_mul(ec, l2));
        }
        const int* id = kSplitOrd[sp.lo][sp.hi];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          double o[6];
#pragma unroll
          for (int k = 0; k < 6; ++k) o[k] = __ldg(rec + 3 * id[k] + c);
          const double pV = g.V * o[0] + g.E * o[3] + g.C * o[5];
          const double pE = g.E * o[1] + g.V * o[3] + g.C * o[4];
          const double pC = g.C * o[2] + g.E * o[4] + g.V * o[5];
          P[c] = g.V * pV + g.E * pE + g.C * pC;
          const ff fV = ff_of(pV), fE = ff_of(pE), fC = ff_of(pC);
          w.set(c, ff_dot3(fV, w.get(6), fE, w.get(7), fC, w.get(8)));
          w.set(3 + c, ff_dot3(fV, w.get(9), fE, w.get(10), fC, w.get(11)));
        }
        ++since;
      } else {
        Ords<3> o;
        load_ords<3>(rec, sp, o);
        sbb<3>(o, g, P);
      }
      }
      // Location, barycentrics and sub-triangle choice are invariant under
      // p -> lambda p (lambda > 0) and the patch is homogeneous of degree 2,
      // so the projection onto the sphere can wait: normalising every
      // kNormEvery-th submap (and the result) keeps |p| within ~1e-3 of 1
      // for queries on the sphere (|P| = 1 + O(h^3) per submap, the
      // deviation at most doubled per submap) and saves the FP64 square
      // root and scaling.  The tangent pushes then carry exactly the factor
      // |p| / 2^(submaps since the last normalisation) against the
      // normalised chain, and their components along p stay along p
      // (DP(p)[p] = 2 P); both are removed where the point is normalised.
      if ((s & (kNormEvery - 1)) != 0) {
        p[0] = P[0];
        p[1] = P[1];
        p[2] = P[2];
        continue;
      }
      const double inv_n = rsqrt(P[0] * P[0] + P[1] * P[1] + P[2] * P[2]);
      p[0] = P[0] * inv_n;
      p[1] = P[1] * inv_n;
      p[2] = P[2] * inv_n;
      if (JAC) {
        const ff sc = ff_of(inv_n * pow2(since));
        since = 0;
        const ff u0 = ff_of(p[0]), u1 = ff_of(p[1]), u2 = ff_of(p[2]);
        const ff d1 = ff_dot3(u0, w.get(0), u1, w.get(1), u2, w.get(2));
        const ff d2 = ff_dot3(u0, w.get(3), u1, w.get(4), u2, w.get(5));
        const ff u[3] = {u0, u1, u2};
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          w.set(c, ff_mul(ff_sub(w.get(c), ff_mul(u[c], d1)), sc));
          w.set(3 + c, ff_mul(ff_sub(w.get(3 + c), ff_mul(u[c], d2)), sc));
        }
      }
    }
    if (!finite3(p[0], p[1], p[2])) flag(m, CMM_FLAG_NONFINITE);
    out[3 * i] = p[0];
    out[3 * i + 1] = p[1];
    out[3 * i + 2] = p[2];
    if (JAC) {
      // the basis again, from q re-read (cheaper than keeping it in
      // registers across the submap loop)
      const double q0[3] = {q[3 * i], q[3 * i + 1], q[3 * i + 2]};
      ff t1[3], t2[3];
      tangent_basis_ff(q0, t1, t2);
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b2 = 0; b2 < 3; ++b2)
          jac[9 * i + 3 * a + b2] = ff_to_double(ff_dot2(w.get(a), t1[b2], w.get(3 + a), t2[b2]));
    }
  }
}

__global__ void __launch_bounds__(kBlock) stencil_kernel(MeshView m, const double* __restrict__ coeffs,
                                                         const double* __restrict__ yn,
                                                         const double* __restrict__ st, int64_t nv,
                                                         double* __restrict__ out) {
  const int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (v >= nv) return;
  const double x = yn[v], y = yn[nv + v], z = yn[2 * nv + v];
  if (!finite3(x, y, z)) {
    flag(m, CMM_FLAG_NONFINITE);
    for (int k = 0; k < 12; ++k) out[k * nv + v] = nan("");
    return;
  }
  const int t = locate_row(m, x, y, z);
  double Lr[13];
  load_loc(m, t, Lr);
  const Split sp = split_of(bcc_of(Lr, x, y, z));
  Ords<3> o;
  load_ords<3>(coeffs + (int64_t)t * kCoeffStride3, sp, o);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const double sx = st[(0 * 4 + k) * nv + v], sy = st[(1 * 4 + k) * nv + v],
                 sz = st[(2 * 4 + k) * nv + v];
    const Gam g = gamma_of(Lr, bcc_of(Lr, sx, sy, sz), sp);
    double P[3];
    sbb<3>(o, g, P);
#pragma unroll
    for (int c = 0; c < 3; ++c) out[(c * 4 + k) * nv + v] = P[c];
  }
}

// ------------------------------------------------------- query order
// Counting sort of the queries by coarse cell (the hierarchy node of level
// kOrderLevel containing the query, FP32 descent, no FP64 filter: any
// cell is a valid bucket) in four passes without global atomics:
// per-block histograms, a scan along each cell's row of blocks, a scan of
// the cell totals, a scatter.
constexpr int kOrderLevel = 4;          // 20 * 4^4 = 5120 cells
constexpr int kOrderCells = 20 << (2 * kOrderLevel);
constexpr int kOrderBlock = 1024;       // threads per block of passes 1 and 3
constexpr int kOrderPer = 16;           // queries per thread

__device__ __forceinline__ int coarse_cell(const MeshView& m, double x, double y, double z) {
  const float fx = (float)x, fy = (float)y, fz = (float)z;
  const float* rf = m.root_f;
  int f = 0;
  float best = -4.0f;
  for (int g = 0; g < 20; ++g) {
    const float d = fmaf(rf[12 * g], fx, fmaf(rf[12 * g + 1], fy, rf[12 * g + 2] * fz));
    if (d > best) {
      best = d;
      f = g;
    }
  }
  int64_t off = 0, cnt = 20;
  const int lv = m.level < kOrderLevel ? m.level : kOrderLevel;
  for (int j = 0; j < lv; ++j) {
    const float* nf = m.node_nf + 9 * (off + f);
    int c;
    if (plane_f(nf, fx, fy, fz) > 0.f) c = 0;
    else if (plane_f(nf + 3, fx, fy, fz) > 0.f) c = 1;
    else if (plane_f(nf + 6, fx, fy, fz) > 0.f) c = 2;
    else c = 3;
    off += cnt;
    cnt *= 4;
    f = 4 * f + c;
  }
  return f << (2 * (kOrderLevel - lv));
}

// pass 1: keys and per-block histograms hist[cell * nblk + block]
__global__ void __launch_bounds__(kOrderBlock) order_count_kernel(MeshView m, const double* __restrict__ q,
                                                                  int64_t n, int32_t* __restrict__ key,
                                                                  int32_t* __restrict__ hist) {
  __shared__ int h[kOrderCells];
  for (int k = threadIdx.x; k < kOrderCells; k += blockDim.x) h[k] = 0;
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * kOrderBlock * kOrderPer;
  for (int r = 0; r < kOrderPer; ++r) {
    const int64_t i = base + (int64_t)r * kOrderBlock + threadIdx.x;
    if (i < n) {
      const int c = coarse_cell(m, q[3 * i], q[3 * i + 1], q[3 * i + 2]);
      key[i] = c;
      atomicAdd(&h[c], 1);
    }
  }
  __syncthreads();
  for (int k = threadIdx.x; k < kOrderCells; k += blockDim.x) hist[(int64_t)k * gridDim.x + blockIdx.x] = h[k];
}

// pass 2: per cell (one warp each) the exclusive scan of its row of block
// counts in place, and the cell total
__global__ void __launch_bounds__(256) order_rowscan_kernel(int32_t* __restrict__ hist, int nblk,
                                                            int32_t* __restrict__ total) {
  const int c = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (c >= kOrderCells) return;
  int32_t* row = hist + (int64_t)c * nblk;
  int carry = 0;
  for (int b0 = 0; b0 < nblk; b0 += 32) {
    const int b = b0 + lane;
    const int v = b < nblk ? row[b] : 0;
    int inc = v;
    for (int d = 1; d < 32; d <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, inc, d);
      if (lane >= d) inc += t;
    }
    if (b < nblk) row[b] = carry + inc - v;
    carry += __shfl_sync(0xffffffffu, inc, 31);
  }
  if (lane == 0) total[c] = carry;
}

// pass 3: exclusive scan of the cell totals (one block)
__global__ void __launch_bounds__(1024) order_cellscan_kernel(int32_t* __restrict__ total) {
  constexpr int per = (kOrderCells + 1023) / 1024;
  __shared__ int part[1024];
  const int lo = threadIdx.x * per;
  int v[per], s = 0;
  for (int k = 0; k < per; ++k) {
    v[k] = lo + k < kOrderCells ? total[lo + k] : 0;
    s += v[k];
  }
  part[threadIdx.x] = s;
  __syncthreads();
  for (int d = 1; d < 1024; d <<= 1) {
    const int t = threadIdx.x >= d ? part[threadIdx.x - d] : 0;
    __syncthreads();
    part[threadIdx.x] += t;
    __syncthreads();
  }
  int acc = part[threadIdx.x] - s;
  for (int k = 0; k < per; ++k)
    if (lo + k < kOrderCells) {
      total[lo + k] = acc;
      acc += v[k];
    }
}

// pass 4: scatter the query ids into their cells' ranges
__global__ void __launch_bounds__(kOrderBlock) order_scatter_kernel(const int32_t* __restrict__ key, int64_t n,
                                                                    const int32_t* __restrict__ hist,
                                                                    const int32_t* __restrict__ cbase,
                                                                    int32_t* __restrict__ perm) {
  __shared__ int h[kOrderCells];
  for (int k = threadIdx.x; k < kOrderCells; k += blockDim.x)
    h[k] = cbase[k] + hist[(int64_t)k * gridDim.x + blockIdx.x];
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * kOrderBlock * kOrderPer;
  for (int r = 0; r < kOrderPer; ++r) {
    const int64_t i = base + (int64_t)r * kOrderBlock + threadIdx.x;
    if (i < n) perm[atomicAdd(&h[key[i]], 1)] = (int32_t)i;
  }
}

// Cube-map jump table: the row containing every cell centre, by the
// hierarchy descent (the view passed has no jump table yet).
__global__ void __launch_bounds__(kBlock) jump_table_kernel(MeshView m, int R, int* __restrict__ table) {
  const int64_t n = 6LL * R * R;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
    const int face = (int)(c / ((int64_t)R * R)), iv = (int)((c / R) % R), iu = (int)(c % R);
    const double u = -1.0 + (iu + 0.5) * 2.0 / R, v = -1.0 + (iv + 0.5) * 2.0 / R;
    const double sg = (face & 1) ? -1.0 : 1.0;
    double d[3];
    if (face < 2) {
      d[0] = sg; d[1] = u; d[2] = v;
    } else if (face < 4) {
      d[0] = u; d[1] = sg; d[2] = v;
    } else {
      d[0] = u; d[1] = v; d[2] = sg;
    }
    const double in = 1.0 / sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    table[c] = locate_descent(m, d[0] * in, d[1] * in, d[2] * in);
  }
}

int check_launch(const char* what) {
  note_launch();
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? CMM_OK : cuda_fail(e, what);
}

}  // namespace

int launch_locate(const MeshView& m, const double* q, int64_t n, int32_t* tri, double* bcc,
                  cudaStream_t s) {
  if (n == 0) return CMM_OK;
  const int b = block_for(m, kTuneLocate, kBlock, n);
  locate_kernel<<<grid_for(n, b), b, 0, s>>>(m, q, n, tri, bcc);
  return check_launch("locate_kernel");
}

int launch_assemble(const MeshView& m, const double* jets, int ncomp, double* coeffs,
                    cudaStream_t s, const BveState* st) {
  const int blocks = (m.nt + kAsmTri - 1) / kAsmTri;
  if (ncomp == 3 && m.rec32)
    assemble_f32_kernel<double><<<blocks, kAsmTri, 0, s>>>(m, jets, (float*)coeffs, st);
  else if (ncomp == 3)
    assemble_kernel<3><<<blocks, kAsmTri, 0, s>>>(m, jets, coeffs, st);
  else
    assemble_kernel<1><<<blocks, kAsmTri, 0, s>>>(m, jets, coeffs, st);
  return check_launch("assemble_kernel");
}

int launch_assemble_f32_jets(const MeshView& m, const float* jets, cudaStream_t s, const BveState* st) {
  if (!m.rec32 || !st) {
    set_last_error("assemble from FP32 jets: FP32 records and a device-driven state expected");
    return CMM_ERR_ARG;
  }
  const int blocks = (m.nt + kAsmTri - 1) / kAsmTri;
  assemble_f32_kernel<float><<<blocks, kAsmTri, 0, s>>>(m, jets, nullptr, st);
  return check_launch("assemble_f32_kernel");
}

int launch_compose(const MeshView& m, const double* const* coeffs, int S, const double* q,
                   int64_t n, double* out, int32_t* tri, int32_t* tri_all, double* jac,
                   cudaStream_t s, const int32_t* perm, const double* const* forms,
                   const float* const* forms_ff) {
  if (n == 0) return CMM_OK;
  SubmapPtrs cp;
  cp.S = S;
  // the float-float copies are used when every submap with a form record
  // has one
  bool ff = forms_ff != nullptr;
  for (int k = 0; k < S; ++k) {
    cp.p[k] = coeffs[k];
    cp.f[k] = forms ? forms[k] : nullptr;
    cp.g[k] = forms && forms[k] && forms_ff ? forms_ff[k] : nullptr;
    if (cp.f[k] && !cp.g[k]) ff = false;
  }
  const int b = block_for(m, kTuneCompose, kBlock, n);
  const int g = grid_for(n, b);
  if (jac) {
    const int v = m.variant[CMM_VARIANT_COMPOSE_JAC] ? m.variant[CMM_VARIANT_COMPOSE_JAC]
                                                    : (ff ? kComposeJacBlocksFF : kComposeJacBlocks);
    if (v == 2 && ff)
      compose_kernel<true, SubmapPtrs, 2, true><<<g, b, 0, s>>>(m, cp, q, n, out, tri, tri_all, jac, perm);
    else if (v == 2)
      compose_kernel<true, SubmapPtrs, 2><<<g, b, 0, s>>>(m, cp, q, n, out, tri, tri_all, jac, perm);
    else if (v == 3 && ff)
      compose_kernel<true, SubmapPtrs, 3, true><<<g, b, 0, s>>>(m, cp, q, n, out, tri, tri_all, jac, perm);
    else if (v == 3)
      compose_kernel<true, SubmapPtrs, 3><<<g, b, 0, s>>>(m, cp, q, n, out, tri, tri_all, jac, perm);
    else if (ff)
      compose_kernel<true, SubmapPtrs, 4, true><<<g, b, 0, s>>>(m, cp, q, n, out, tri, tri_all, jac, perm);
    else
      compose_kernel<true, SubmapPtrs, 4><<<g, b, 0, s>>>(m, cp, q, n, out, tri, tri_all, jac, perm);
  } else if ((m.variant[CMM_VARIANT_COMPOSE] ? m.variant[CMM_VARIANT_COMPOSE] : kComposeBlocks) == 4) {
    compose_kernel<false, SubmapPtrs, 4><<<g, b, 0, s>>>(m, cp, q, n, out, tri, tri_all, jac, perm);
  } else {
    compose_kernel<false, SubmapPtrs, 6><<<g, b, 0, s>>>(m, cp, q, n, out, tri, tri_all, jac, perm);
  }
  return check_launch("compose_kernel");
}

int launch_assemble_forms(const MeshView& m, const double* coeffs, double* forms, cudaStream_t s) {
  const int64_t n = 6LL * m.nt;
  assemble_forms_kernel<<<(int)((n + 127) / 128), 128, 0, s>>>(m, coeffs, forms);
  return check_launch("assemble_forms_kernel");
}

int launch_forms_ff(const MeshView& m, const double* forms, float* forms_ff, cudaStream_t s) {
  const int64_t n = 18LL * m.nt;
  forms_ff_kernel<<<(int)((n + 127) / 128), 128, 0, s>>>(m.nt, forms, forms_ff);
  return check_launch("forms_ff_kernel");
}

int launch_remap_forms(const MeshView& m, const BveState* st, int n_maps, int Nt, const double* const* table,
                       double* const* ftable, cudaStream_t s) {
  const int64_t n = 6LL * m.nt;
  remap_forms_kernel<<<(int)((n + 127) / 128), 128, 0, s>>>(m, st, n_maps, Nt, table, ftable);
  return check_launch("remap_forms_kernel");
}

int make_asm_f32(cmm_mesh* mesh) {
  const int64_t n = (int64_t)kAsmFactors * mesh->view.nt;
  const int64_t nl = (int64_t)kLocStride * mesh->view.nt;
  int rc = mesh->tri_asm_f.alloc(n * sizeof(float));
  if (rc || (rc = mesh->tri_loc_f.alloc(nl * sizeof(float)))) return rc;
  to_f32_kernel<<<(int)((n + 255) / 256), 256>>>(mesh->view.tri_asm, n, (float*)mesh->tri_asm_f.p);
  if ((rc = check_launch("to_f32_kernel"))) return rc;
  to_f32_kernel<<<(int)((nl + 255) / 256), 256>>>(mesh->view.tri_loc, nl, (float*)mesh->tri_loc_f.p);
  if ((rc = check_launch("to_f32_kernel"))) return rc;
  cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return cuda_fail(e, "make_asm_f32");
  mesh->view.tri_asm_f = (const float*)mesh->tri_asm_f.p;
  mesh->view.tri_loc_f = (const float*)mesh->tri_loc_f.p;
  return CMM_OK;
}

int build_jump_table(cmm_mesh* mesh) {
  MeshView& v = mesh->view;
  const int R = std::min(1024, std::max(16, 4 << v.level));
  const int64_t n = 6LL * R * R;
  int rc = mesh->jump.alloc(n * sizeof(int));
  if (rc) return rc;
  MeshView m = v;
  m.jump = nullptr;
  jump_table_kernel<<<grid_for(n, kBlock), kBlock>>>(m, R, (int*)mesh->jump.p);
  if ((rc = check_launch("jump_table_kernel"))) return rc;
  cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return cuda_fail(e, "build_jump_table");
  v.jump = (const int*)mesh->jump.p;
  v.jump_res = R;
  return CMM_OK;
}

int64_t order_workspace(int64_t n) {
  const int64_t nblk = (n + (int64_t)kOrderBlock * kOrderPer - 1) / ((int64_t)kOrderBlock * kOrderPer);
  return n + (int64_t)kOrderCells * ((nblk < 1 ? 1 : nblk) + 1);
}

int launch_query_order(const MeshView& m, const double* q, int64_t n, int32_t* perm, int32_t* work,
                       cudaStream_t s) {
  if (n == 0) return CMM_OK;
  const int64_t nblk = (n + (int64_t)kOrderBlock * kOrderPer - 1) / ((int64_t)kOrderBlock * kOrderPer);
  int32_t* key = work;
  int32_t* hist = work + n;
  int32_t* total = hist + (int64_t)kOrderCells * nblk;
  order_count_kernel<<<(int)nblk, kOrderBlock, 0, s>>>(m, q, n, key, hist);
  int rc = check_launch("order_count_kernel");
  if (rc) return rc;
  order_rowscan_kernel<<<kOrderCells / 8, 256, 0, s>>>(hist, (int)nblk, total);
  if ((rc = check_launch("order_rowscan_kernel"))) return rc;
  order_cellscan_kernel<<<1, 1024, 0, s>>>(total);
  if ((rc = check_launch("order_cellscan_kernel"))) return rc;
  order_scatter_kernel<<<(int)nblk, kOrderBlock, 0, s>>>(key, n, hist, total, perm);
  return check_launch("order_scatter_kernel");
}

int launch_compose_dev(const MeshView& m, const double* const* table, const BveState* st,
                       const double* last, const double* q, int64_t n, double* out, cudaStream_t s,
                       const double* const* ftable) {
  if (n == 0) return CMM_OK;
  DevSubmaps cp{table, ftable, st, last};
  const int b = block_for(m, kTuneCompose, kBlock, n);
  if ((m.variant[CMM_VARIANT_COMPOSE] ? m.variant[CMM_VARIANT_COMPOSE] : kComposeBlocks) == 4)
    compose_kernel<false, DevSubmaps, 4><<<grid_for(n, b), b, 0, s>>>(m, cp, q, n, out, nullptr, nullptr,
                                                                      nullptr, nullptr);
  else
    compose_kernel<false, DevSubmaps, 6><<<grid_for(n, b), b, 0, s>>>(m, cp, q, n, out, nullptr, nullptr,
                                                                      nullptr, nullptr);
  return check_launch("compose_kernel");
}

int launch_stencil_eval(const MeshView& m, const double* coeffs, const double* yn,
                        const double* st, int64_t nv, double* out, cudaStream_t s) {
  if (nv == 0) return CMM_OK;
  stencil_kernel<<<(int)((nv + kBlock - 1) / kBlock), kBlock, 0, s>>>(m, coeffs, yn, st, nv, out);
  return check_launch("stencil_kernel");
}

}  // namespace cmm
