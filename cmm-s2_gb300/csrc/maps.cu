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

#include "cmm_internal.h"
#include "geom.h"

namespace cmm {

__constant__ SplitTables c_split;

namespace {

constexpr float kFilter = 1e-6f;
constexpr int kBlock = 256;

struct SubmapPtrs {
  const double* p[CMM_MAX_SUBMAPS];
};

// FP32-filtered sign test of n.q; returns the FP64 dot when undecided.
__device__ __forceinline__ bool plane_pos(const float* nf, const double* nd, float qx, float qy,
                                          float qz, double dx, double dy, double dz) {
  float t = fmaf(nf[0], qx, fmaf(nf[1], qy, nf[2] * qz));
  if (fabsf(t) > kFilter) return t > 0.0f;
  double td = nd[0] * dx + nd[1] * dy + nd[2] * dz;
  return td > 0.0;
}

__device__ __forceinline__ float plane_f(const float* nf, float qx, float qy, float qz) {
  return fmaf(nf[0], qx, fmaf(nf[1], qy, nf[2] * qz));
}

// Reference row of the triangle containing q.
__device__ __forceinline__ int locate_row(const MeshView& m, double x, double y, double z) {
  const float fx = (float)x, fy = (float)y, fz = (float)z;
  // root face: nearest face centre (FP32), then exact edge checks with a
  // bounded walk across the violated edge
  const float* rf = m.root_f;
  int f = 0;
  float best = -4.0f;
#pragma unroll 4
  for (int g = 0; g < 20; ++g) {
    float d = fmaf(rf[12 * g], fx, fmaf(rf[12 * g + 1], fy, rf[12 * g + 2] * fz));
    if (d > best) {
      best = d;
      f = g;
    }
  }
  for (int it = 0; it < 6; ++it) {
    int e = -1;
    for (int k = 0; k < 3; ++k) {
      const float* nf = rf + 12 * f + 3 + 3 * k;
      float t = plane_f(nf, fx, fy, fz);
      bool neg;
      if (fabsf(t) > kFilter) {
        neg = t < 0.0f;
      } else {
        const double* nd = m.root + 12 * f + 3 + 3 * k;
        neg = (nd[0] * x + nd[1] * y + nd[2] * z) < 0.0;
      }
      if (neg) {
        e = k;
        break;
      }
    }
    if (e < 0) break;
    const int g2 = m.root_adj[3 * f + e];
    if (g2 < 0 || g2 >= 20) break;
    f = g2;
  }
  // descent
  int64_t off = 0, cnt = 20;
  for (int j = 0; j < m.level; ++j) {
    const int64_t node = off + f;
    const float* nf = m.node_nf + 9 * node;
    const double* nd = m.node_n + 9 * node;
    int c;
    if (plane_pos(nf, nd, fx, fy, fz, x, y, z))
      c = 0;
    else if (plane_pos(nf + 3, nd + 3, fx, fy, fz, x, y, z))
      c = 1;
    else if (plane_pos(nf + 6, nd + 6, fx, fy, fz, x, y, z))
      c = 2;
    else
      c = 3;
    off += cnt;
    cnt *= 4;
    f = 4 * f + c;
  }
  return __ldg(m.leaf_row + f);
}

struct Bcc {
  double b0, b1, b2;
};

__device__ __forceinline__ Bcc bcc_of(const double* L, double x, double y, double z) {
  return Bcc{L[0] * x + L[1] * y + L[2] * z, L[3] * x + L[4] * y + L[5] * z,
             L[6] * x + L[7] * y + L[8] * z};
}

// Powell-Sabin sub-triangle of a big-triangle bcc: lo/hi with numpy's
// first-occurrence rule; when all three are equal (the split centre) the
// reference's table has no sub-triangle (it yields 0/0); any sub-triangle
// is exact there, (lo,hi) = (1,0) is used.
struct Split {
  int lo, mid, hi;
};

__device__ __forceinline__ Split split_of(const Bcc& b) {
  int lo = 0, hi = 0;
  double vlo = b.b0, vhi = b.b0;
  if (b.b1 < vlo) { vlo = b.b1; lo = 1; }
  if (b.b2 < vlo) { vlo = b.b2; lo = 2; }
  if (b.b1 > vhi) { vhi = b.b1; hi = 1; }
  if (b.b2 > vhi) { vhi = b.b2; hi = 2; }
  if (lo == hi) { lo = 1; hi = 0; }
  return Split{lo, 3 - lo - hi, hi};
}

__device__ __forceinline__ double pick(const Bcc& b, int i) {
  return i == 0 ? b.b0 : (i == 1 ? b.b1 : b.b2);
}

// Edge-midpoint norm |v_hi + v_mid| from the location record.
__device__ __forceinline__ double edge_norm(const double* L, int a, int b) {
  int s = a + b;  // {0,1}->1 N12, {1,2}->3 N23, {0,2}->2 N31
  return s == 1 ? L[10] : (s == 3 ? L[11] : L[12]);
}

struct Gam {
  double V, E, C;
};

__device__ __forceinline__ Gam gamma_of(const double* L, const Bcc& b, const Split& sp) {
  double bl = pick(b, sp.lo), bm = pick(b, sp.mid), bh = pick(b, sp.hi);
  return Gam{bh - bm, edge_norm(L, sp.hi, sp.mid) * (bm - bl), L[9] * bl};
}

// Six ordinates x ncomp of the sub-triangle, canonical order
// V^2, E^2, C^2, VE, EC, VC.
template <int NC>
struct Ords {
  double c[6][NC];
};

template <int NC>
__device__ __forceinline__ void load_ords(const double* rec, const Split& sp, Ords<NC>& o) {
  const int* id = c_split.ord[sp.lo][sp.hi];
#pragma unroll
  for (int k = 0; k < 6; ++k)
#pragma unroll
    for (int c = 0; c < NC; ++c) o.c[k][c] = __ldg(rec + NC * id[k] + c);
}

template <int NC>
__device__ __forceinline__ void sbb(const Ords<NC>& o, const Gam& g, double* P) {
  const double vv = g.V * g.V, ee = g.E * g.E, cc = g.C * g.C;
  const double ve = 2 * g.V * g.E, ec = 2 * g.E * g.C, vc = 2 * g.V * g.C;
#pragma unroll
  for (int c = 0; c < NC; ++c)
    P[c] = vv * o.c[0][c] + ee * o.c[1][c] + cc * o.c[2][c] + ve * o.c[3][c] + ec * o.c[4][c] +
           vc * o.c[5][c];
}

// Tangent image of w under one normalised submap: dS = (dP - s (s.dP)) / |P|.
__device__ __forceinline__ void push_tangent(const double* L, const Split& sp, const Gam& g,
                                             const Ords<3>& o, const double* s, double inv_n,
                                             double* w) {
  const Bcc d = bcc_of(L, w[0], w[1], w[2]);
  const double dl = pick(d, sp.lo), dm = pick(d, sp.mid), dh = pick(d, sp.hi);
  double dV = dh - dm, dE = edge_norm(L, sp.hi, sp.mid) * (dm - dl), dC = L[9] * dl;
  double dP[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    double pV = g.V * o.c[0][c] + g.E * o.c[3][c] + g.C * o.c[5][c];
    double pE = g.E * o.c[1][c] + g.V * o.c[3][c] + g.C * o.c[4][c];
    double pC = g.C * o.c[2][c] + g.E * o.c[4][c] + g.V * o.c[5][c];
    dP[c] = 2 * (pV * dV + pE * dE + pC * dC);
  }
  double sd = s[0] * dP[0] + s[1] * dP[1] + s[2] * dP[2];
#pragma unroll
  for (int c = 0; c < 3; ++c) w[c] = (dP[c] - s[c] * sd) * inv_n;
}

__device__ __forceinline__ void flag(const MeshView& m, int bit) { atomicOr(m.status, bit); }

__global__ void __launch_bounds__(kBlock) locate_kernel(MeshView m, const double* __restrict__ q,
                                                        int64_t n, int32_t* __restrict__ tri,
                                                        double* __restrict__ bcc) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double x = q[3 * i], y = q[3 * i + 1], z = q[3 * i + 2];
    if (!(isfinite(x) && isfinite(y) && isfinite(z))) {
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

template <int NC>
__global__ void __launch_bounds__(128) assemble_kernel(MeshView m, const double* __restrict__ jets,
                                                       double* __restrict__ coeffs, int stride) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= m.nt) return;
  const int nv = m.nv;
  const int4 tv = m.tri_v[t];
  const int vid[3] = {tv.x, tv.y, tv.z};
  const double* A = m.tri_asm + (int64_t)t * kAsmStride;
  double* out = coeffs + (int64_t)t * stride;
  // ordinates 3..11: (corner, factor slot)
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
      const double* a = A + 4 * o;
      c[3 + o] = a[0] * gx + a[1] * gy + a[2] * gz - a[3] * f[corner[o]];
    }
    c[12] = A[36] * c[3] + A[37] * c[8];
    c[13] = A[38] * c[6] + A[39] * c[11];
    c[14] = A[41] * c[9] + A[40] * c[5];
    c[15] = A[36] * c[4] + A[37] * c[7];
    c[16] = A[38] * c[7] + A[39] * c[10];
    c[17] = A[40] * c[4] + A[41] * c[10];
    c[18] = A[42] * c[4] + A[43] * c[7] + A[44] * c[10];
#pragma unroll
    for (int o = 0; o < 19; ++o) out[NC * o + k] = c[o];
  }
}

template <bool JAC>
__global__ void __launch_bounds__(kBlock) compose_kernel(MeshView m, SubmapPtrs cp, int S,
                                                         const double* __restrict__ q, int64_t n,
                                                         double* __restrict__ out,
                                                         int32_t* __restrict__ tri,
                                                         int32_t* __restrict__ tri_all,
                                                         double* __restrict__ jac) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double p[3] = {q[3 * i], q[3 * i + 1], q[3 * i + 2]};
    if (!(isfinite(p[0]) && isfinite(p[1]) && isfinite(p[2]))) {
      flag(m, CMM_FLAG_NONFINITE);
      out[3 * i] = out[3 * i + 1] = out[3 * i + 2] = nan("");
      if (tri) tri[i] = -1;
      if (tri_all)
        for (int s = 0; s < S; ++s) tri_all[(int64_t)s * n + i] = -1;
      if (JAC)
        for (int k = 0; k < 9; ++k) jac[9 * i + k] = nan("");
      continue;
    }
    double t1[3], t2[3], w1[3], w2[3];
    if (JAC) {  // orthonormal tangent basis at q
      double ax = fabs(p[2]) < 0.9 ? 0.0 : 1.0, az = 1.0 - ax;
      t1[0] = p[1] * az;
      t1[1] = p[2] * ax - p[0] * az;
      t1[2] = -p[1] * ax;
      double in = rsqrt(t1[0] * t1[0] + t1[1] * t1[1] + t1[2] * t1[2]);
      t1[0] *= in; t1[1] *= in; t1[2] *= in;
      t2[0] = p[1] * t1[2] - p[2] * t1[1];
      t2[1] = p[2] * t1[0] - p[0] * t1[2];
      t2[2] = p[0] * t1[1] - p[1] * t1[0];
      for (int c = 0; c < 3; ++c) { w1[c] = t1[c]; w2[c] = t2[c]; }
    }
    for (int s = S - 1; s >= 0; --s) {
      const int t = locate_row(m, p[0], p[1], p[2]);
      if (s == S - 1 && tri) tri[i] = t;
      if (tri_all) tri_all[(int64_t)s * n + i] = t;
      const double* L = m.tri_loc + (int64_t)t * kLocStride;
      double Lr[13];
#pragma unroll
      for (int k = 0; k < 13; ++k) Lr[k] = __ldg(L + k);
      const Bcc b = bcc_of(Lr, p[0], p[1], p[2]);
      const Split sp = split_of(b);
      const Gam g = gamma_of(Lr, b, sp);
      Ords<3> o;
      load_ords<3>(cp.p[s] + (int64_t)t * kCoeffStride3, sp, o);
      double P[3];
      sbb<3>(o, g, P);
      const double inv_n = rsqrt(P[0] * P[0] + P[1] * P[1] + P[2] * P[2]);
      double sN[3] = {P[0] * inv_n, P[1] * inv_n, P[2] * inv_n};
      if (JAC) {
        push_tangent(Lr, sp, g, o, sN, inv_n, w1);
        push_tangent(Lr, sp, g, o, sN, inv_n, w2);
      }
      p[0] = sN[0];
      p[1] = sN[1];
      p[2] = sN[2];
    }
    if (!(isfinite(p[0]) && isfinite(p[1]) && isfinite(p[2]))) flag(m, CMM_FLAG_NONFINITE);
    out[3 * i] = p[0];
    out[3 * i + 1] = p[1];
    out[3 * i + 2] = p[2];
    if (JAC) {
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b2 = 0; b2 < 3; ++b2) jac[9 * i + 3 * a + b2] = w1[a] * t1[b2] + w2[a] * t2[b2];
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
  if (!(isfinite(x) && isfinite(y) && isfinite(z))) {
    flag(m, CMM_FLAG_NONFINITE);
    for (int k = 0; k < 12; ++k) out[k * nv + v] = nan("");
    return;
  }
  const int t = locate_row(m, x, y, z);
  const double* L = m.tri_loc + (int64_t)t * kLocStride;
  double Lr[13];
#pragma unroll
  for (int k = 0; k < 13; ++k) Lr[k] = __ldg(L + k);
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

int grid_for(int64_t n, int block) {
  int64_t b = (n + block - 1) / block;
  const int64_t cap = 152LL * 16;
  return (int)(b < cap ? (b < 1 ? 1 : b) : cap);
}

}  // namespace

void upload_split_tables_host(SplitTables* t) {
  // reference tables (cmm_s2/core/spherical_spline.py:660-666)
  static const int ords[3][3][6] = {{{0, 0, 0, 0, 0, 0}, {18, 1, 13, 7, 6, 16}, {13, 2, 18, 11, 10, 16}},
                                    {{18, 14, 0, 17, 5, 4}, {0, 0, 0, 0, 0, 0}, {14, 18, 2, 17, 10, 9}},
                                    {{0, 12, 18, 3, 15, 4}, {1, 18, 12, 7, 15, 8}, {0, 0, 0, 0, 0, 0}}};
  static const int corners[3][3][3] = {{{0, 0, 0}, {3, 1, 5}, {5, 2, 3}},
                                       {{3, 6, 0}, {0, 0, 0}, {6, 3, 2}},
                                       {{0, 4, 3}, {1, 3, 4}, {0, 0, 0}}};
  for (int lo = 0; lo < 3; ++lo)
    for (int hi = 0; hi < 3; ++hi) {
      for (int k = 0; k < 6; ++k) t->ord[lo][hi][k] = 0;
      if (lo == hi) continue;
      int pv = -1, pe = -1, pc = -1;
      for (int p = 0; p < 3; ++p) {
        int c = corners[lo][hi][p];
        if (c == hi) pv = p;
        else if (c == 3) pc = p;
        else pe = p;
      }
      const int* o = ords[lo][hi];
      auto pair = [&](int a, int b) {
        int s = a + b;  // {0,1}->o[3], {1,2}->o[4], {0,2}->o[5]
        return s == 1 ? o[3] : (s == 3 ? o[4] : o[5]);
      };
      t->ord[lo][hi][0] = o[pv];
      t->ord[lo][hi][1] = o[pe];
      t->ord[lo][hi][2] = o[pc];
      t->ord[lo][hi][3] = pair(pv, pe);
      t->ord[lo][hi][4] = pair(pe, pc);
      t->ord[lo][hi][5] = pair(pv, pc);
    }
}

int set_split_tables() {
  SplitTables t;
  upload_split_tables_host(&t);
  cudaError_t e = cudaMemcpyToSymbol(c_split, &t, sizeof(t));
  return e == cudaSuccess ? CMM_OK : cuda_fail(e, "cudaMemcpyToSymbol(split tables)");
}

static int check_launch(const char* what) {
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? CMM_OK : cuda_fail(e, what);
}

int launch_locate(const MeshView& m, const double* q, int64_t n, int32_t* tri, double* bcc,
                  cudaStream_t s) {
  if (n == 0) return CMM_OK;
  locate_kernel<<<grid_for(n, kBlock), kBlock, 0, s>>>(m, q, n, tri, bcc);
  return check_launch("locate_kernel");
}

int launch_assemble(const MeshView& m, const double* jets, int ncomp, double* coeffs,
                    cudaStream_t s) {
  const int blocks = (m.nt + 127) / 128;
  if (ncomp == 3)
    assemble_kernel<3><<<blocks, 128, 0, s>>>(m, jets, coeffs, kCoeffStride3);
  else
    assemble_kernel<1><<<blocks, 128, 0, s>>>(m, jets, coeffs, kCoeffStride1);
  return check_launch("assemble_kernel");
}

int launch_compose(const MeshView& m, const double* const* coeffs, int S, const double* q,
                   int64_t n, double* out, int32_t* tri, int32_t* tri_all, double* jac,
                   cudaStream_t s) {
  if (n == 0) return CMM_OK;
  SubmapPtrs cp;
  for (int k = 0; k < S; ++k) cp.p[k] = coeffs[k];
  const int g = grid_for(n, kBlock);
  if (jac)
    compose_kernel<true><<<g, kBlock, 0, s>>>(m, cp, S, q, n, out, tri, tri_all, jac);
  else
    compose_kernel<false><<<g, kBlock, 0, s>>>(m, cp, S, q, n, out, tri, tri_all, jac);
  return check_launch("compose_kernel");
}

int launch_stencil_eval(const MeshView& m, const double* coeffs, const double* yn,
                        const double* st, int64_t nv, double* out, cudaStream_t s) {
  if (nv == 0) return CMM_OK;
  stencil_kernel<<<(int)((nv + kBlock - 1) / kBlock), kBlock, 0, s>>>(m, coeffs, yn, st, nv, out);
  return check_launch("stencil_kernel");
}

}  // namespace cmm
