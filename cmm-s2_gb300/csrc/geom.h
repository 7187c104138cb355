// Small FP64 vector geometry shared by host set-up code and kernels.
#pragma once
#include <math.h>

#ifdef __CUDACC__
#define CMM_HD __host__ __device__ __forceinline__
#else
#define CMM_HD inline
#endif

namespace cmm {

struct D3 {
  double x, y, z;
};

CMM_HD D3 d3(double x, double y, double z) { return D3{x, y, z}; }
CMM_HD D3 operator+(D3 a, D3 b) { return D3{a.x + b.x, a.y + b.y, a.z + b.z}; }
CMM_HD D3 operator-(D3 a, D3 b) { return D3{a.x - b.x, a.y - b.y, a.z - b.z}; }
CMM_HD D3 operator*(double s, D3 a) { return D3{s * a.x, s * a.y, s * a.z}; }
CMM_HD D3 operator/(D3 a, double s) { return D3{a.x / s, a.y / s, a.z / s}; }
CMM_HD double dot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
CMM_HD D3 cross(D3 a, D3 b) {
  return D3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
CMM_HD double norm(D3 a) { return sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
// Row normalisation as utils.div_norm (cmm_s2/core/utils.py:36-38).
CMM_HD D3 unit(D3 a) {
  double n = sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
  return D3{a.x / n, a.y / n, a.z / n};
}
// Determinant of the matrix with columns a, b, c: the six-term expansion
// of utils.det_vec (cmm_s2/core/utils.py:49-56).
CMM_HD double det_cols(D3 a, D3 b, D3 c) {
  return a.x * b.y * c.z + b.x * c.y * a.z + a.y * b.z * c.x -
         (c.x * b.y * a.z + c.y * b.z * a.x + b.x * a.y * c.z);
}
// Un-normalised spherical barycentrics of q in (v1,v2,v3) (utils.py:58-67).
CMM_HD D3 bary(D3 v1, D3 v2, D3 v3, D3 q) {
  double d = det_cols(v1, v2, v3);
  return D3{det_cols(q, v2, v3) / d, det_cols(v1, q, v3) / d, det_cols(v1, v2, q) / d};
}
// Unit tangent projection of a at the unit point b
// (mesh_functions.sphere_tan_proj, cmm_s2/core/mesh_functions.py:320-329).
CMM_HD D3 tan_unit(D3 a, D3 b) {
  double c = dot(b, a);
  double d = sqrt(dot(a, a) - 2 * c * c + dot(b, b) * c * c);
  return D3{(a.x - c * b.x) / d, (a.y - c * b.y) / d, (a.z - c * b.z) / d};
}

// Assembly factors of one triangle (kAsmStride doubles) from its corners,
// following the Powell-Sabin split of ps_split
// (cmm_s2/core/mesh_functions.py:92-126) and the ordinate formulas of
// assemble_coefficients (cmm_s2/core/spherical_spline.py:300-337).
CMM_HD void assembly_factors(D3 v1, D3 v2, D3 v3, double* f) {
  D3 v4 = unit((v1 + v2 + v3) / 3.0);
  D3 e1 = unit(0.5 * v1 + 0.5 * v2), e2 = unit(0.5 * v2 + 0.5 * v3), e3 = unit(0.5 * v3 + 0.5 * v1);
  D3 h12 = tan_unit(v2 - v1, v1), h21 = tan_unit(v1 - v2, v2), h23 = tan_unit(v3 - v2, v2);
  D3 h32 = tan_unit(v2 - v3, v3), h13 = tan_unit(v3 - v1, v1), h31 = tan_unit(v1 - v3, v3);
  D3 h41 = tan_unit(v4 - v1, v1), h42 = tan_unit(v4 - v2, v2), h43 = tan_unit(v4 - v3, v3);
  D3 g12 = bary(v1, e1, v4, h12), g21 = bary(v2, v4, e1, h21);
  D3 g23 = bary(v2, e2, v4, h23), g32 = bary(v3, v4, e2, h32);
  D3 g13 = bary(v1, v4, e3, h13), g31 = bary(v3, e3, v4, h31);
  D3 g14 = bary(v1, v4, e3, tan_unit(v4, v1));
  D3 g24 = bary(v2, v4, e1, tan_unit(v4, v2));
  D3 g34 = bary(v3, v4, e2, tan_unit(v4, v3));
  D3 mid = bary(v1, v2, v3, v4);
  D3 E0 = bary(v1, v2, v3, e1), E1 = bary(v1, v2, v3, e2), E2 = bary(v1, v2, v3, e3);
  // ordinates 3..11: (h, g, divisor component)
  const D3 hs[9] = {h12, h41, h13, h23, h42, h21, h31, h43, h32};
  const D3 gs[9] = {g12, g14, g13, g23, g24, g21, g31, g34, g32};
  const int dc[9] = {1, 1, 2, 1, 1, 2, 1, 1, 2};
  for (int k = 0; k < 9; ++k) {
    double g0 = gs[k].x, gd = dc[k] == 1 ? gs[k].y : gs[k].z;
    f[4 * k + 0] = hs[k].x / (2 * gd);
    f[4 * k + 1] = hs[k].y / (2 * gd);
    f[4 * k + 2] = hs[k].z / (2 * gd);
    f[4 * k + 3] = g0 / gd;
  }
  f[36] = E0.x;
  f[37] = E0.y;
  f[38] = E1.y;
  f[39] = E1.z;
  f[40] = E2.x;
  f[41] = E2.z;
  f[42] = mid.x;
  f[43] = mid.y;
  f[44] = mid.z;
  f[45] = f[46] = f[47] = 0.0;
}

// Location record of one triangle (kLocStride doubles).
CMM_HD void location_record(D3 v1, D3 v2, D3 v3, double* r) {
  double d = det_cols(v1, v2, v3);
  D3 r1 = cross(v2, v3) / d, r2 = cross(v3, v1) / d, r3 = cross(v1, v2) / d;
  r[0] = r1.x; r[1] = r1.y; r[2] = r1.z;
  r[3] = r2.x; r[4] = r2.y; r[5] = r2.z;
  r[6] = r3.x; r[7] = r3.y; r[8] = r3.z;
  r[9] = norm(v1 + v2 + v3);
  r[10] = norm(v1 + v2);
  r[11] = norm(v2 + v3);
  r[12] = norm(v3 + v1);
  r[13] = r[14] = r[15] = 0.0;
}

}  // namespace cmm
