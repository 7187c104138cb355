// Device helpers shared by the kernel translation units: icosahedral point
// location, barycentrics, Powell-Sabin sub-triangle selection and the
// quadratic Bernstein-Bezier patch.
#pragma once
#include <cuda_runtime.h>

#include "cmm_internal.h"
#include "geom.h"

namespace cmm {
namespace dev {

constexpr float kFilter = 1e-6f;

// Ordinates of the quadratic patch of each Powell-Sabin sub-triangle in the
// sub-triangle's own corners -- V the triangle vertex with the largest
// barycentric, E the midpoint of the edge from V to the middle vertex, C
// the split centre -- in the order V^2, E^2, C^2, 2VE, 2EC, 2VC; indexed
// [argmin][argmax].  Derived from the reference's ordinate and corner
// tables (cmm_s2/core/spherical_spline.py:660-666) by re-ordering each
// entry's corners (tests/test_host_abi.py re-derives it).
__constant__ const int kSplitOrd[3][3][6] = {
    {{0, 0, 0, 0, 0, 0}, {1, 13, 18, 6, 16, 7}, {2, 13, 18, 11, 16, 10}},
    {{0, 14, 18, 5, 17, 4}, {0, 0, 0, 0, 0, 0}, {2, 14, 18, 9, 17, 10}},
    {{0, 12, 18, 3, 15, 4}, {1, 12, 18, 8, 15, 7}, {0, 0, 0, 0, 0, 0}}};

__device__ __forceinline__ float plane_f(const float* nf, float qx, float qy, float qz) {
  return fmaf(nf[0], qx, fmaf(nf[1], qy, nf[2] * qz));
}

// FP32-filtered sign test of n.q > 0 (FP64 when |n.q| < kFilter).
__device__ __forceinline__ bool plane_pos(const float* nf, const double* nd, float qx, float qy,
                                          float qz, double dx, double dy, double dz) {
  float t = plane_f(nf, qx, qy, qz);
  if (fabsf(t) > kFilter) return t > 0.0f;
  double td = nd[0] * dx + nd[1] * dy + nd[2] * dz;
  return td > 0.0;
}

// x as a float truncated toward zero (0 below 2^-126; |x| < 2^128), from
// its bit pattern on the integer pipe: a rounding conversion would occupy
// the FP64 pipe, the one that bounds the composition.  Within one FP32 ulp
// of x, which the filter bound kFilter covers with margin.
__device__ __forceinline__ float to_f32_trunc(double x) {
  const long long b = __double_as_longlong(x);
  const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
  const unsigned mag = hi & 0x7fffffffu;
  const unsigned f = mag < (897u << 20) ? 0u : (((mag - (896u << 20)) << 3) | (lo >> 29));
  return __uint_as_float((hi & 0x80000000u) | f);
}

// Reference row of the icosahedral triangle containing q, by descent of
// the refinement hierarchy (20 root faces, then one of four children per
// level).
__device__ __forceinline__ int locate_descent(const MeshView& m, double x, double y, double z) {
  const float fx = to_f32_trunc(x), fy = to_f32_trunc(y), fz = to_f32_trunc(z);
  // root face: nearest face centre (FP32), then exact edge checks with a
  // bounded walk across a violated edge
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

// Cell of the cube-map jump table containing the direction (x, y, z): the
// face of the dominant axis, then R x R cells over the two other
// coordinates divided by the dominant one.  Approximate arithmetic is
// enough (the walk starts from any row); every input, NaN included, maps to
// a valid cell.
__device__ __forceinline__ int jump_cell(int R, float x, float y, float z) {
  const float ax = fabsf(x), ay = fabsf(y), az = fabsf(z);
  int face;
  float u, v, den;
  if (ax >= ay && ax >= az) {
    face = x >= 0.f ? 0 : 1;
    u = y;
    v = z;
    den = ax;
  } else if (ay >= az) {
    face = y >= 0.f ? 2 : 3;
    u = x;
    v = z;
    den = ay;
  } else {
    face = z >= 0.f ? 4 : 5;
    u = x;
    v = y;
    den = az;
  }
  const float sc = __fdividef(0.5f * (float)R, den);
  const int iu = min(max((int)((u + den) * sc), 0), R - 1);
  const int iv = min(max((int)((v + den) * sc), 0), R - 1);
  return (face * R + iv) * R + iu;
}

// FP32 side value of q against edge k's unit normal, and the decision
// "q strictly outside edge k of row t": the FP32 sign, redone in FP64
// within the filter.  The row across the edge holds the exactly negated
// normals, so two rows never both reject q.
__device__ __forceinline__ float edge_dot(float4 e, float fx, float fy, float fz) {
  return fmaf(e.x, fx, fmaf(e.y, fy, e.z * fz));
}

__device__ __forceinline__ bool edge_out(const MeshView& m, int t, int k, float d, double x, double y, double z) {
  if (fabsf(d) > kFilter) return d < 0.0f;
  const double* n = m.walk_d + (int64_t)t * kWalkStride + 3 * k;
  return n[0] * x + n[1] * y + n[2] * z < 0.0;
}

// Walk from the jump-table row of q's cube-map cell across the first edge
// that q lies outside of until q is inside all three (a handful of steps:
// the cells are smaller than the triangles).  Returns the row, with the
// three FP32 edge values of the final row in d, or -1 after kWalkMax steps.
__device__ __forceinline__ int walk_locate(const MeshView& m, double x, double y, double z, float fx, float fy,
                                           float fz, float* d) {
  int t = __ldg(m.jump + jump_cell(m.jump_res, fx, fy, fz));
  for (int it = 0; it < kWalkMax; ++it) {
    const float4* r = reinterpret_cast<const float4*>(m.walk_f + (int64_t)t * kWalkStride);
    const float4 e0 = __ldg(r), e1 = __ldg(r + 1), e2 = __ldg(r + 2);
    d[0] = edge_dot(e0, fx, fy, fz);
    d[1] = edge_dot(e1, fx, fy, fz);
    d[2] = edge_dot(e2, fx, fy, fz);
    if (edge_out(m, t, 0, d[0], x, y, z))
      t = __float_as_int(e0.w);
    else if (edge_out(m, t, 1, d[1], x, y, z))
      t = __float_as_int(e1.w);
    else if (edge_out(m, t, 2, d[2], x, y, z))
      t = __float_as_int(e2.w);
    else
      return t;
  }
  return -1;
}

// Reference row of the icosahedral triangle containing q.  With the jump
// table built: the walk, falling back to the hierarchy descent if it has
// not ended after kWalkMax steps.  Both are exact containment tests, so
// they agree except for queries within rounding distance of an edge,
// where either neighbour contains the query.
__device__ __forceinline__ int locate_row(const MeshView& m, double x, double y, double z) {
  if (!m.jump) return locate_descent(m, x, y, z);
  float d[3];
  const int t = walk_locate(m, x, y, z, to_f32_trunc(x), to_f32_trunc(y), to_f32_trunc(z), d);
  return t >= 0 ? t : locate_descent(m, x, y, z);
}

struct Bcc {
  double b0, b1, b2;
};

__device__ __forceinline__ Bcc bcc_of(const double* L, double x, double y, double z) {
  return Bcc{L[0] * x + L[1] * y + L[2] * z, L[3] * x + L[4] * y + L[5] * z,
             L[6] * x + L[7] * y + L[8] * z};
}

// Powell-Sabin sub-triangle of a big-triangle bcc: lo/hi with numpy's
// first-occurrence rule (cmm_s2/core/spherical_spline.py:691-697).  When
// all three are equal (the split centre) the reference's tables select no
// sub-triangle (it returns 0/0); every sub-triangle is exact there and
// (lo,hi) = (1,0) is used.
struct Split {
  int lo, mid, hi;
};

// A signed integer with the order of the double x (-0 and +0 equal):
// +|bits| or -|bits| of its magnitude.  Comparisons of these keys run on
// the integer pipe and give exactly the FP64 comparisons of finite values,
// which would occupy the FP64 pipe (a NaN orders as a large magnitude; the
// split it selects is still one of the six).
__device__ __forceinline__ long long ord_key(double x) {
  const long long b = __double_as_longlong(x);
  const long long mag = b & 0x7fffffffffffffffLL;
  return b < 0 ? -mag : mag;
}

__device__ __forceinline__ Split split_of(const Bcc& b) {
  const long long k0 = ord_key(b.b0), k1 = ord_key(b.b1), k2 = ord_key(b.b2);
  int lo = 0, hi = 0;
  long long vlo = k0, vhi = k0;
  if (k1 < vlo) { vlo = k1; lo = 1; }
  if (k2 < vlo) { vlo = k2; lo = 2; }
  if (k1 > vhi) { vhi = k1; hi = 1; }
  if (k2 > vhi) { vhi = k2; hi = 2; }
  if (lo == hi) { lo = 1; hi = 0; }
  return Split{lo, 3 - lo - hi, hi};
}

// Row containing q and its Powell-Sabin sub-triangle.  The barycentrics
// come in FP32 from the walk's final edge values (b_i = s_i d), and their
// order decides the sub-triangle when every pair is farther apart than
// the sum of their FP32 error bounds (s_i kFilter); otherwise -- and when
// the walk fell back to the descent -- the FP64 barycentrics R q decide,
// with split_of's rule.  Either way the choice is split_of(R q)'s.
__device__ __forceinline__ int locate_split(const MeshView& m, double x, double y, double z, Split* sp) {
  int t = -1;
  if (m.jump) {
    float d[3];
    t = walk_locate(m, x, y, z, to_f32_trunc(x), to_f32_trunc(y), to_f32_trunc(z), d);
    if (t >= 0) {
      const float4 sc = __ldg(reinterpret_cast<const float4*>(m.walk_f + (int64_t)t * kWalkStride) + 3);
      const float b0 = sc.x * d[1], b1 = sc.y * d[2], b2 = sc.z * d[0];
      const float e0 = sc.x * kFilter, e1 = sc.y * kFilter, e2 = sc.z * kFilter;
      if (fabsf(b0 - b1) > e0 + e1 && fabsf(b1 - b2) > e1 + e2 && fabsf(b0 - b2) > e0 + e2) {
        const int lo = b0 < b1 ? (b0 < b2 ? 0 : 2) : (b1 < b2 ? 1 : 2);
        const int hi = b0 > b1 ? (b0 > b2 ? 0 : 2) : (b1 > b2 ? 1 : 2);
        *sp = Split{lo, 3 - lo - hi, hi};
        return t;
      }
    }
  }
  if (t < 0) t = locate_descent(m, x, y, z);
  const double* L = m.tri_loc + (int64_t)t * kLocStride;
  double R[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) R[k] = __ldg(L + k);
  *sp = split_of(bcc_of(R, x, y, z));
  return t;
}

// Index of a sub-triangle (lo, hi), lo != hi, in a map-form record, and
// the inverse tables.
__constant__ const int kSubIndex[3][3] = {{0, 0, 1}, {2, 0, 3}, {4, 5, 0}};
__constant__ const int kSubLo[6] = {0, 0, 1, 1, 2, 2};
__constant__ const int kSubHi[6] = {1, 2, 0, 2, 0, 1};

__device__ __forceinline__ double pick(const Bcc& b, int i) {
  return i == 0 ? b.b0 : (i == 1 ? b.b1 : b.b2);
}

// Edge-midpoint norm |v_a + v_b| from the location record.
__device__ __forceinline__ double edge_norm(const double* L, int a, int b) {
  int s = a + b;  // {0,1}->N12, {1,2}->N23, {0,2}->N31
  return s == 1 ? L[10] : (s == 3 ? L[11] : L[12]);
}

struct Gam {
  double V, E, C;
};

// Sub-triangle barycentrics from the big-triangle ones (closed form; the
// sub-triangle's corners are v_hi, (v_hi+v_mid)/|.|, (v1+v2+v3)/|.|).
__device__ __forceinline__ Gam gamma_of(const double* L, const Bcc& b, const Split& sp) {
  double bl = pick(b, sp.lo), bm = pick(b, sp.mid), bh = pick(b, sp.hi);
  return Gam{bh - bm, edge_norm(L, sp.hi, sp.mid) * (bm - bl), L[9] * bl};
}

// FP32 barycentrics, sub-triangle and sub-triangle barycentrics from the
// FP32 location record (velocity patches of the mixed form; the patch is
// C1 across sub-triangles, so an FP32 ordering of nearly equal
// barycentrics changes the value at rounding level only).
struct BccF {
  float b0, b1, b2;
};

__device__ __forceinline__ BccF bcc_of_f(const float* L, float x, float y, float z) {
  return BccF{fmaf(L[0], x, fmaf(L[1], y, L[2] * z)), fmaf(L[3], x, fmaf(L[4], y, L[5] * z)),
              fmaf(L[6], x, fmaf(L[7], y, L[8] * z))};
}

// b = Minv p = Minv (p - v1) + (1, 0, 0): the difference p - v1 (size of
// the triangle) is formed in FP64 and the FP32 product then carries no
// cancellation (Minv's rows are ~1/h long; Minv p in FP32 would lose
// h^-1 * 6e-8 of b).
__device__ __forceinline__ BccF bcc_rel_f(const MeshView& m, int t, const float* L, double x, double y,
                                          double z) {
  const int v1 = __ldg(&m.tri_v[t].x);
  const double* v = m.verts + 4 * (int64_t)v1;
  const float dx = to_f32_trunc(x - __ldg(v)), dy = to_f32_trunc(y - __ldg(v + 1)),
              dz = to_f32_trunc(z - __ldg(v + 2));
  BccF b = bcc_of_f(L, dx, dy, dz);
  b.b0 += 1.0f;
  return b;
}

__device__ __forceinline__ Split split_of_f(const BccF& b) {
  int lo = 0, hi = 0;
  float vlo = b.b0, vhi = b.b0;
  if (b.b1 < vlo) { vlo = b.b1; lo = 1; }
  if (b.b2 < vlo) { vlo = b.b2; lo = 2; }
  if (b.b1 > vhi) { vhi = b.b1; hi = 1; }
  if (b.b2 > vhi) { vhi = b.b2; hi = 2; }
  if (lo == hi) { lo = 1; hi = 0; }
  return Split{lo, 3 - lo - hi, hi};
}

__device__ __forceinline__ float pick_f(const BccF& b, int i) {
  return i == 0 ? b.b0 : (i == 1 ? b.b1 : b.b2);
}

__device__ __forceinline__ void gamma_of_f(const float* L, const BccF& b, const Split& sp, float* g) {
  const float bl = pick_f(b, sp.lo), bm = pick_f(b, sp.mid), bh = pick_f(b, sp.hi);
  const int s = sp.hi + sp.mid;
  const float en = s == 1 ? L[10] : (s == 3 ? L[11] : L[12]);
  g[0] = bh - bm;
  g[1] = en * (bm - bl);
  g[2] = L[9] * bl;
}

template <int NC>
struct Ords {
  double c[6][NC];
};

template <int NC>
__device__ __forceinline__ void load_ords(const double* rec, const Split& sp, Ords<NC>& o) {
  const int* id = kSplitOrd[sp.lo][sp.hi];
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

// FP32 velocity records: the six ordinates of the sub-triangle and the
// patch in FP32 (the barycentrics and sub-triangle choice stay FP64).
template <int NC>
struct OrdsF {
  float c[6][NC];
};

template <int NC>
__device__ __forceinline__ void load_ords_f(const float* rec, const Split& sp, OrdsF<NC>& o) {
  const int* id = kSplitOrd[sp.lo][sp.hi];
#pragma unroll
  for (int k = 0; k < 6; ++k)
#pragma unroll
    for (int c = 0; c < NC; ++c) o.c[k][c] = __ldg(rec + NC * id[k] + c);
}

template <int NC>
__device__ __forceinline__ void sbb_f(const OrdsF<NC>& o, float V, float E, float C, float* P) {
  const float vv = V * V, ee = E * E, cc = C * C;
  const float ve = 2 * V * E, ec = 2 * E * C, vc = 2 * V * C;
#pragma unroll
  for (int c = 0; c < NC; ++c)
    P[c] = vv * o.c[0][c] + ee * o.c[1][c] + cc * o.c[2][c] + ve * o.c[3][c] + ec * o.c[4][c] +
           vc * o.c[5][c];
}

__device__ __forceinline__ void load_loc(const MeshView& m, int t, double* Lr) {
  const double* L = m.tri_loc + (int64_t)t * kLocStride;
#pragma unroll
  for (int k = 0; k < 13; ++k) Lr[k] = __ldg(L + k);
}

__device__ __forceinline__ void flag(const MeshView& m, int bit) { atomicOr(m.status, bit); }

__device__ __forceinline__ bool finite3(double x, double y, double z) {
  return isfinite(x) && isfinite(y) && isfinite(z);
}

constexpr double kTwoPi = 6.283185307179586;

// numpy float floor_divide / remainder for b > 0 (npy_divmod): exact fmod,
// then the quotient of the exact difference, rounded to the nearest
// integer below.
__device__ __forceinline__ double np_floor_divide(double a, double b) {
  double mod = fmod(a, b);
  double div = (a - mod) / b;
  if (mod != 0.0 && (mod < 0.0)) div -= 1.0;
  if (div == 0.0) return copysign(0.0, a / b);
  double fl = floor(div);
  if (div - fl > 0.5) fl += 1.0;
  return fl;
}

__device__ __forceinline__ double np_remainder(double a, double b) {
  double mod = fmod(a, b);
  if (mod != 0.0) {
    if (mod < 0.0) mod += b;
  } else {
    mod = copysign(0.0, b);
  }
  return mod;
}

// utils.cart2sphere (cmm_s2/core/utils.py:18-23): phi in [0, 2 pi), theta.
__device__ __forceinline__ void cart2sphere(double x, double y, double z, double* phi,
                                            double* theta) {
  *phi = np_remainder(atan2(y, x) + kTwoPi, kTwoPi);
  *theta = atan2(sqrt(__dadd_rn(__dmul_rn(y, y), __dmul_rn(x, x))), z);
}

// ------------------------------------------------ lat-lon velocity mesh
__device__ __forceinline__ int py_mod(long long a, int n) {
  long long r = a % n;
  return (int)(r < 0 ? r + n : r);
}

// With g(ring, p) the ring points: g(ring, p) x g(ring, p+1) (ring edge)
// and g(ring, p) x g(ring+1, p+1) (cell diagonal), from the mesh's tables
// (numpy's rounding).
__device__ __forceinline__ D3 table_normal(const double* tab, const MeshView& m, int ring, int p) {
  const double2* e = reinterpret_cast<const double2*>(tab + 4 * ((int64_t)ring * 2 * m.L + p));
  const double2 a = __ldg(e), b = __ldg(e + 1);
  return D3{a.x, a.y, b.x};
}
__device__ __forceinline__ D3 ring_normal(const MeshView& m, int ring, int p) {
  return table_normal(m.ring_n, m, ring, p);
}
__device__ __forceinline__ D3 diag_normal(const MeshView& m, int ring, int p) {
  return table_normal(m.diag_n, m, ring, p);
}

// Triangle (row of the lat-lon table) containing q: ring and sector from
// the angles with numpy's floor-division semantics, the reference's
// near-row corrections and the diagonal side test
// (structure_spherical_triangulation.inds / containing_simplex_and_bcc_structured,
// cmm_s2/core/mesh_functions.py:201-282).
static __device__ __noinline__ int latlon_locate_exact(const MeshView& m, double x, double y, double z) {
  const int N = 2 * m.L, M = m.L + 1;
  double phi = np_remainder(atan2(y, x) + kTwoPi, kTwoPi);
  const double rho = sqrt(__dadd_rn(__dmul_rn(y, y), __dmul_rn(x, x)));
  const double theta = atan2(rho, z);
  const double phiq = np_remainder(phi, kTwoPi);
  const int phi_l = py_mod((long long)np_floor_divide(phiq - m.phi[0], m.dphi), N);
  int theta_l = (int)np_floor_divide(theta - m.theta[0], m.dthe);
  if (theta_l == M - 1) theta_l = M - 2;
  if (theta_l < 0) theta_l = 0;
  if (theta_l > M - 2) theta_l = M - 2;
  const double theta_c = (theta - m.theta[theta_l]) / m.dthe;
  const D3 q = D3{x, y, z};
  const bool row_lo = theta_c <= 0.03 && theta_l != 0;
  const bool row_hi = !row_lo && theta_c > 0.85 && theta_l != M - 2;
  if (row_lo || row_hi) {
    // the reference tests the point re-synthesised from its angles,
    // sphere2cart(phi, theta) (mesh_functions.py:240, 249)
    double sp, cp, st, cth;
    sincos(phiq, &sp, &cp);
    sincos(theta, &st, &cth);
    const D3 q0 = D3{st * cp, st * sp, cth};
    if (row_lo) {
      const D3 n = ring_normal(m, theta_l, phi_l);
      if (dot(n, q0) > 0.0) theta_l -= 1;
    } else {
      const D3 n = ring_normal(m, theta_l + 1, phi_l);
      if (-dot(n, q0) > 0.0) theta_l += 1;
    }
  }
  if (theta_l == 0) return phi_l;
  if (theta_l == M - 2) return 2 * N * (M - 2) - N + phi_l;
  const D3 n = diag_normal(m, theta_l, phi_l);
  const int s = (-dot(n, q) > 0.0) ? 1 : 0;
  return N + 2 * (N * (theta_l - 1) + phi_l) + s;
}

// The same location with the angles taken in FP32 (FP64 atan2/fmod cost
// ~100 FP64 instructions on a part whose FP64 rate is 1/58 of FP32): the
// cell indices and the row-correction thresholds are read off the FP32
// angles when every fractional part is farther than the FP32 error bound
// (2e-6 rad, scaled to cell units) from a decision boundary; the sign tests
// then run in FP64 against q and are trusted when |n.q| > 1e-13 (the
// re-synthesised point q0 of the reference differs from q by ~1e-16).
// Otherwise the exact FP64 path decides, so both give the same triangle.
__device__ __forceinline__ int latlon_locate(const MeshView& m, double x, double y, double z) {
  const int N = 2 * m.L, M = m.L + 1;
  const float xf = to_f32_trunc(x), yf = to_f32_trunc(y), zf = to_f32_trunc(z);
  float phif = atan2f(yf, xf);
  if (phif < 0.f) phif += 6.28318530717958647692f;
  const float thef = atan2f(sqrtf(xf * xf + yf * yf), zf);
  const float u = (phif - m.phi0_f) / m.dphi_f;
  const float v = (thef - m.the0_f) / m.dthe_f;
  const float du = 2e-6f / m.dphi_f, dv = 2e-6f / m.dthe_f;
  const float uf = floorf(u), vf = floorf(v);
  const float fu = u - uf, fv = v - vf;
  const int phi_l = (int)uf;
  int theta_l = (int)vf;
  if (!(fu > du && fu < 1.f - du && fv > dv && fv < 1.f - dv && fabsf(fv - 0.03f) > dv &&
        fabsf(fv - 0.85f) > dv && phi_l >= 0 && phi_l < N && theta_l >= 0 && theta_l <= M - 2))
    return latlon_locate_exact(m, x, y, z);
  const D3 q = D3{x, y, z};
  const bool row_lo = fv <= 0.03f && theta_l != 0;
  const bool row_hi = !row_lo && fv > 0.85f && theta_l != M - 2;
  if (row_lo) {
    const double d = dot(ring_normal(m, theta_l, phi_l), q);
    if (fabs(d) <= 1e-13) return latlon_locate_exact(m, x, y, z);
    if (d > 0.0) theta_l -= 1;
  } else if (row_hi) {
    const double d = -dot(ring_normal(m, theta_l + 1, phi_l), q);
    if (fabs(d) <= 1e-13) return latlon_locate_exact(m, x, y, z);
    if (d > 0.0) theta_l += 1;
  }
  if (theta_l == 0) return phi_l;
  if (theta_l == M - 2) return 2 * N * (M - 2) - N + phi_l;
  const D3 n = diag_normal(m, theta_l, phi_l);
  const int s = (-dot(n, q) > 0.0) ? 1 : 0;
  return N + 2 * (N * (theta_l - 1) + phi_l) + s;
}

// Scalar Powell-Sabin spline (ncomp = 1 coefficients) on the lat-lon mesh
// at q (spherical_spline.__call__, cmm_s2/core/spherical_spline.py:42-70).
__device__ __forceinline__ double latlon_scalar(const MeshView& m, const double* __restrict__ coeffs,
                                                double x, double y, double z) {
  const int t = latlon_locate(m, x, y, z);
  double Lr[13];
  load_loc(m, t, Lr);
  const Bcc b = bcc_of(Lr, x, y, z);
  const Split sp = split_of(b);
  const Gam g = gamma_of(Lr, b, sp);
  Ords<1> o;
  load_ords<1>(coeffs + (int64_t)t * kCoeffStride1, sp, o);
  double P[1];
  sbb<1>(o, g, P);
  return P[0];
}

// Real orthonormal spherical-harmonic series (coefficients (lmax+1,
// 2 lmax+1), column l+m: m = 0 -> Pbar_l0, m > 0 -> sqrt2 Pbar_lm cos(m phi),
// m < 0 -> sqrt2 Pbar_l|m| sin(|m| phi)) at the point (x, y, z), from the
// velocity mesh's recurrence table, cos/sin(m phi) by rotation, no
// transcendental calls.  NS series (coefficient arrays K = (lmax+1)(2lmax+1)
// apart) share the Legendre recurrence.  lmax <= kShTableMax.
struct ShPoint {
  double ct, st, cp, sp;
};

// (reciprocal norms from the FP64 rsqrt, within 1 ulp: square roots and
// divisions would cost ~60 FP64-pipe instructions per point)
__device__ __forceinline__ ShPoint sh_point(double x, double y, double z) {
  const double rho2 = x * x + y * y;
  const double ir = rsqrt(rho2 + z * z);
  ShPoint p;
  p.ct = z * ir;
  if (rho2 > 0.0) {
    const double irho = rsqrt(rho2);
    p.st = rho2 * irho * ir;
    p.cp = x * irho;
    p.sp = y * irho;
  } else {   // atan2(0, 0) = 0
    p.st = 0.0;
    p.cp = 1.0;
    p.sp = 0.0;
  }
  return p;
}

template <int NS>
__device__ __forceinline__ void sh_series_n(const MeshView& vm, const double* __restrict__ c, int lmax,
                                            const ShPoint& pt, double* out) {
  const int T = kShTableMax + 1;
  const int w = 2 * lmax + 1;
  const int64_t K = (int64_t)(lmax + 1) * w;
#pragma unroll
  for (int k = 0; k < NS; ++k) out[k] = 0.0;
  double pmm = 0.28209479177387814;   // sqrt(1/(4 pi))
  double cm = 1.0, sm = 0.0;          // cos(m phi), sin(m phi)
  for (int m = 0; m <= lmax; ++m) {
    if (m > 0) {
      pmm = -pmm * __ldg(vm.sh_fm + m) * pt.st;
      const double c2 = cm * pt.cp - sm * pt.sp;
      sm = sm * pt.cp + cm * pt.sp;
      cm = c2;
    }
    const double* ab = vm.sh_ab + 2 * (int64_t)m * T;
    double p1 = 0.0, p = pmm;
    // sum_l Pbar_lm (c_l,m cos + c_l,-m sin) = cos * sum_l Pbar_lm c_l,m +
    // sin * sum_l Pbar_lm c_l,-m: two FMAs per degree, the angle once per m
    double ac[NS], as[NS];
#pragma unroll
    for (int k = 0; k < NS; ++k) ac[k] = as[k] = 0.0;
    for (int l = m; l <= lmax; ++l) {
      if (l == m + 1) {
        p1 = p;
        p = __ldg(ab + 2 * l) * pt.ct * pmm;
      } else if (l > m + 1) {
        const double pn = __ldg(ab + 2 * l) * (pt.ct * p - __ldg(ab + 2 * l + 1) * p1);
        p1 = p;
        p = pn;
      }
      const int64_t i = (int64_t)l * w + l;
#pragma unroll
      for (int k = 0; k < NS; ++k) {
        ac[k] += c[k * K + i + m] * p;
        if (m > 0) as[k] += c[k * K + i - m] * p;
      }
    }
#pragma unroll
    for (int k = 0; k < NS; ++k)
      out[k] += m == 0 ? ac[k] : 1.4142135623730951 * (ac[k] * cm + as[k] * sm);
  }
}

// The scalar spline in FP32 (mixed form, field32 with FP32 location
// records): FP32 barycentrics and patch from the FP64 ordinates.
__device__ __forceinline__ double latlon_scalar_f(const MeshView& m, const double* __restrict__ coeffs,
                                                  double x, double y, double z) {
  const int t = latlon_locate(m, x, y, z);
  const float* Lf = m.tri_loc_f + (int64_t)t * kLocStride;
  float Lr[13];
#pragma unroll
  for (int k = 0; k < 13; ++k) Lr[k] = __ldg(Lf + k);
  const BccF b = bcc_rel_f(m, t, Lr, x, y, z);
  const Split sp = split_of_f(b);
  float g[3];
  gamma_of_f(Lr, b, sp, g);
  const int* id = kSplitOrd[sp.lo][sp.hi];
  const double* rec = coeffs + (int64_t)t * kCoeffStride1;
  float o[6];
#pragma unroll
  for (int k = 0; k < 6; ++k) o[k] = to_f32_trunc(__ldg(rec + id[k]));
  const float V = g[0], E = g[1], C = g[2];
  return (double)(V * V * o[0] + E * E * o[1] + C * C * o[2] + 2 * V * E * o[3] + 2 * E * C * o[4] +
                  2 * V * C * o[5]);
}

inline int grid_for(int64_t n, int block) {
  int64_t b = (n + block - 1) / block;
  const int64_t cap = 152LL * 16;
  return (int)(b < cap ? (b < 1 ? 1 : b) : cap);
}

}  // namespace dev
}  // namespace cmm
