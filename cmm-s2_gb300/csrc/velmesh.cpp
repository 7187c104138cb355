// Host-side construction of the MWSS lat-lon velocity mesh
// (structure_spherical_triangulation, cmm_s2/core/mesh_functions.py:169-318)
// and the Lagrange time weights of the velocity interpolant.
#include <cmath>

#include "cmm_internal.h"
#include "geom.h"

namespace cmm {

// Triangle table of the lat-lon mesh in the reference's order
// (grid_assemble, cmm_s2/core/mesh_functions.py:380-412): the north cap
// fan, two triangles per quad row by row, the south cap fan.  N = 2L
// points per ring, M = L+1 rings; vertex 0 is the north pole, ring r
// (1..M-2) holds vertices 1+(r-1)N .. rN, the south pole is last.
void latlon_triangles(int L, std::vector<int4>& tv) {
  const int N = 2 * L, M = L + 1;
  tv.clear();
  tv.reserve((size_t)2 * N * (M - 2));
  for (int i = 0; i < N - 1; ++i) tv.push_back(make_int4(0, i + 1, i + 2, 0));
  tv.push_back(make_int4(0, N, 1, 0));
  for (int i = 0; i < M - 3; ++i)
    for (int j = 1; j <= N; ++j) {
      const int k = j + i * N;
      if (j != N) {
        tv.push_back(make_int4(k, k + N + 1, k + 1, 0));
        tv.push_back(make_int4(k, k + N, k + N + 1, 0));
      } else {
        tv.push_back(make_int4(k, k + 1, i * N + 1, 0));
        tv.push_back(make_int4(k, k + N, k + 1, 0));
      }
    }
  const int nn = (M - 3) * N + 1;
  for (int i = nn; i < nn + N - 1; ++i) tv.push_back(make_int4(i, nn + N, i + 1, 0));
  tv.push_back(make_int4(nn + N - 1, nn + N, nn, 0));
}

int build_latlon(int L, const double* theta, const double* phi, const double* grid,
                 const double* verts, cmm_mesh* m) {
  if (L < 3) {
    set_last_error("cmm_velmesh_create: L must be >= 3");
    return CMM_ERR_ARG;
  }
  const int N = 2 * L, M = L + 1;
  const int nv = 2 + (M - 2) * N;
  std::vector<int4> tv;
  latlon_triangles(L, tv);
  const int nt = (int)tv.size();
  std::vector<double> loc((size_t)nt * kLocStride), asmf((size_t)nt * kAsmStride);
  for (int t = 0; t < nt; ++t) {
    auto V = [&](int i) { return D3{verts[3 * i], verts[3 * i + 1], verts[3 * i + 2]}; };
    D3 v1 = V(tv[t].x), v2 = V(tv[t].y), v3 = V(tv[t].z);
    location_record(v1, v2, v3, &loc[(size_t)t * kLocStride]);
    assembly_factors(v1, v2, v3, &asmf[(size_t)t * kAsmStride]);
  }
  std::vector<double> vpad(4 * (size_t)nv), gpad(4 * (size_t)M * N);
  for (int i = 0; i < nv; ++i)
    for (int c = 0; c < 3; ++c) vpad[4 * i + c] = verts[3 * i + c];
  for (int i = 0; i < M * N; ++i)
    for (int c = 0; c < 3; ++c) gpad[4 * i + c] = grid[(size_t)c * M * N + i];
  int rc, zero = 0;
  if ((rc = m->verts.upload(vpad.data(), vpad.size() * 8))) return rc;
  if ((rc = m->tri_v.upload(tv.data(), tv.size() * sizeof(int4)))) return rc;
  if ((rc = m->tri_loc.upload(loc.data(), loc.size() * 8))) return rc;
  if ((rc = upload_asm_factors(m->tri_asm, asmf, nt))) return rc;
  if ((rc = m->theta.upload(theta, (size_t)M * 8))) return rc;
  if ((rc = m->phi.upload(phi, (size_t)N * 8))) return rc;
  if ((rc = m->grid.upload(gpad.data(), gpad.size() * 8))) return rc;
  {
    // side-test normals of the ring edges and the cell diagonals, each
    // cross-product component a_i b_j - a_j b_i with both products rounded
    // (host code without contraction), as numpy's cross
    std::vector<double> rn(4 * (size_t)M * N, 0.0), dn(4 * (size_t)M * N, 0.0);
    auto G = [&](int ring, int p) { return D3{gpad[4 * ((size_t)ring * N + p)], gpad[4 * ((size_t)ring * N + p) + 1],
                                               gpad[4 * ((size_t)ring * N + p) + 2]}; };
    for (int ring = 0; ring < M; ++ring)
      for (int p = 0; p < N; ++p) {
        const D3 a = G(ring, p), b = G(ring, (p + 1) % N);
        const D3 r = cross(a, b);
        double* o = &rn[4 * ((size_t)ring * N + p)];
        o[0] = r.x;
        o[1] = r.y;
        o[2] = r.z;
        if (ring + 1 < M) {
          const D3 d = cross(a, G(ring + 1, (p + 1) % N));
          double* e = &dn[4 * ((size_t)ring * N + p)];
          e[0] = d.x;
          e[1] = d.y;
          e[2] = d.z;
        }
      }
    if ((rc = m->ring_n.upload(rn.data(), rn.size() * 8))) return rc;
    if ((rc = m->diag_n.upload(dn.data(), dn.size() * 8))) return rc;
  }
  {
    std::vector<double> ct(M);
    for (int t = 0; t < M; ++t) ct[t] = std::cos(theta[t]);
    if ((rc = m->cos_theta.upload(ct.data(), ct.size() * 8))) return rc;
  }
  if ((rc = m->status.upload(&zero, sizeof(int)))) return rc;
  {
    // Pbar_lm recurrence: l = m+1: a = sqrt(2m+3); l >= m+2:
    // a = sqrt((4l^2-1)/(l^2-m^2)), b = sqrt(((l-1)^2-m^2)/(4(l-1)^2-1))
    const int T = kShTableMax + 1;
    std::vector<double> ab((size_t)2 * T * T, 0.0), fm(T, 0.0);
    for (int mm = 0; mm < T; ++mm) {
      if (mm > 0) fm[mm] = std::sqrt((2.0 * mm + 1.0) / (2.0 * mm));
      for (int l = mm + 1; l < T; ++l) {
        double a, b = 0.0;
        if (l == mm + 1) {
          a = std::sqrt(2.0 * mm + 3.0);
        } else {
          a = std::sqrt((4.0 * l * l - 1.0) / ((double)l * l - (double)mm * mm));
          b = std::sqrt(((l - 1.0) * (l - 1.0) - (double)mm * mm) / (4.0 * (l - 1.0) * (l - 1.0) - 1.0));
        }
        ab[2 * ((size_t)mm * T + l)] = a;
        ab[2 * ((size_t)mm * T + l) + 1] = b;
      }
    }
    if ((rc = m->sh_ab.upload(ab.data(), ab.size() * 8))) return rc;
    if ((rc = m->sh_fm.upload(fm.data(), fm.size() * 8))) return rc;
  }
  MeshView& v = m->view;
  v = MeshView{};
  v.kind = kLatLon;
  v.level = -1;
  v.nv = nv;
  v.nt = nt;
  v.L = L;
  v.verts = (const double*)m->verts.p;
  v.tri_v = (const int4*)m->tri_v.p;
  v.tri_loc = (const double*)m->tri_loc.p;
  v.tri_asm = (const double*)m->tri_asm.p;
  v.theta = (const double*)m->theta.p;
  v.phi = (const double*)m->phi.p;
  v.grid = (const double*)m->grid.p;
  v.ring_n = (const double*)m->ring_n.p;
  v.diag_n = (const double*)m->diag_n.p;
  v.status = (int*)m->status.p;
  v.sh_ab = (const double*)m->sh_ab.p;
  v.sh_fm = (const double*)m->sh_fm.p;
  // spacing as the reference computes it (mesh_functions.py:214-215)
  v.dphi = std::fabs(phi[1] - phi[0]);
  v.dthe = std::fabs(theta[1] - theta[0]);
  v.phi0_f = (float)phi[0];
  v.dphi_f = (float)v.dphi;
  v.the0_f = (float)theta[0];
  v.dthe_f = (float)v.dthe;
  return CMM_OK;
}

// Lagrange weights of spline_interp_velocity.__call__
// (cmm_s2/core/spherical_spline.py:596-612): one level -> the level itself;
// two -> linear in tau = (t - ts0)/dt; three -> quadratic on ts0, ts0+dt,
// ts0+2dt.
TimeWeights time_weights(int nvs, double ts0, double dt, const double* times, int ntimes) {
  TimeWeights tw{};
  for (int s = 0; s < ntimes; ++s) {
    const double t = times[s];
    if (nvs == 1) {
      tw.w[s][0] = 1.0;
    } else if (nvs == 2) {
      const double tau = (t - ts0) / dt;
      tw.w[s][0] = 1 - tau;
      tw.w[s][1] = tau;
    } else {
      const double t0 = ts0, t1 = ts0 + dt, t2 = ts0 + 2 * dt;
      tw.w[s][0] = (t - t1) * (t - t2) / (2 * dt * dt);
      tw.w[s][1] = (t - t0) * (t - t2) / (-dt * dt);
      tw.w[s][2] = (t - t0) * (t - t1) / (2 * dt * dt);
    }
  }
  return tw;
}

}  // namespace cmm
