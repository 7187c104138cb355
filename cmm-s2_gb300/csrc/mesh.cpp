// Host-side construction of the icosahedral mesh context: the refinement
// hierarchy used for point location, the leaf -> reference-row permutation
// and the per-row location and assembly tables.
//
// The reference locates queries with Qhull (cmm_s2/core/mesh_functions.py:
// 43, 82) and reports the Delaunay simplex index.  Here the caller's
// triangle table (that same Delaunay order) is taken as given, the
// icosahedral hierarchy is rebuilt from the vertex coordinates, and every
// leaf of the hierarchy is mapped back to its row of the caller's table.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <unordered_map>

#include "cmm_internal.h"
#include "geom.h"

namespace cmm {

namespace {
thread_local std::string g_err;
}

void set_last_error(const std::string& s) { g_err = s; }

static std::atomic<long long> g_launches{0};
void note_launch(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
long long launch_count() { return g_launches.load(std::memory_order_relaxed); }
const char* last_error() { return g_err.c_str(); }

int cuda_fail(cudaError_t e, const char* what) {
  set_last_error(std::string(what) + ": " + cudaGetErrorString(e));
  return CMM_ERR_CUDA;
}

DeviceBuffer::~DeviceBuffer() {
  if (p) cudaFree(p);
}

void DeviceBuffer::release() {
  if (p) cudaFree(p);
  p = nullptr;
  bytes = 0;
}

int DeviceBuffer::alloc(size_t n) {
  if (p) cudaFree(p);
  p = nullptr;
  bytes = n;
  if (n == 0) return CMM_OK;
  cudaError_t e = cudaMalloc(&p, n);
  if (e != cudaSuccess) {
    p = nullptr;
    return cuda_fail(e, "cudaMalloc");
  }
  return CMM_OK;
}

int DeviceBuffer::upload(const void* src, size_t n) {
  int rc = alloc(n);
  if (rc) return rc;
  if (n == 0) return CMM_OK;
  cudaError_t e = cudaMemcpy(p, src, n, cudaMemcpyHostToDevice);
  return e == cudaSuccess ? CMM_OK : cuda_fail(e, "cudaMemcpy");
}

namespace {

// Nearest-vertex lookup on a uniform hash grid.
class VertexGrid {
 public:
  VertexGrid(const double* v, int n, double cell) : v_(v), cell_(cell) {
    for (int i = 0; i < n; ++i) cells_[key(cx(v[3 * i]), cx(v[3 * i + 1]), cx(v[3 * i + 2]))].push_back(i);
  }
  int find(D3 p, double tol) const {
    int ix = cx(p.x), iy = cx(p.y), iz = cx(p.z);
    int best = -1;
    double bd = tol * tol;
    for (int a = -1; a <= 1; ++a)
      for (int b = -1; b <= 1; ++b)
        for (int c = -1; c <= 1; ++c) {
          auto it = cells_.find(key(ix + a, iy + b, iz + c));
          if (it == cells_.end()) continue;
          for (int i : it->second) {
            double dx = v_[3 * i] - p.x, dy = v_[3 * i + 1] - p.y, dz = v_[3 * i + 2] - p.z;
            double d = dx * dx + dy * dy + dz * dz;
            if (d <= bd) {
              bd = d;
              best = i;
            }
          }
        }
    return best;
  }

 private:
  int cx(double x) const { return (int)std::floor(x / cell_); }
  static int64_t key(int64_t a, int64_t b, int64_t c) {
    return ((a + (1 << 20)) << 42) | ((b + (1 << 20)) << 21) | (c + (1 << 20));
  }
  const double* v_;
  double cell_;
  std::unordered_map<int64_t, std::vector<int>> cells_;
};

D3 vtx(const double* v, int i) { return D3{v[3 * i], v[3 * i + 1], v[3 * i + 2]}; }

int64_t tri_key(int a, int b, int c, int64_t nv) {
  int s[3] = {a, b, c};
  std::sort(s, s + 3);
  return ((int64_t)s[0] * nv + s[1]) * nv + s[2];
}

}  // namespace

int build_host(const double* verts, int nv, const int32_t* tris, int nt, int level, HostMesh* hm) {
  if (level < 0 || level > 10) {
    set_last_error("cmm_mesh_create: level must be in [0, 10]");
    return CMM_ERR_ARG;
  }
  const int64_t nt_exp = 20LL << (2 * level), nv_exp = 10LL * (1LL << (2 * level)) + 2;
  if (nt != nt_exp || nv != nv_exp) {
    set_last_error("cmm_mesh_create: sizes do not match an icosahedral refinement of this level");
    return CMM_ERR_MESH;
  }
  for (int64_t i = 0; i < 3LL * nt; ++i)
    if (tris[i] < 0 || tris[i] >= nv) {
      set_last_error("cmm_mesh_create: triangle vertex id out of range");
      return CMM_ERR_ARG;
    }
  // valence: 12 base vertices have 5 incident triangles
  std::vector<int> val(nv, 0);
  for (int64_t i = 0; i < 3LL * nt; ++i) val[tris[i]]++;
  std::vector<int> base;
  for (int i = 0; i < nv; ++i)
    if (val[i] == 5) base.push_back(i);
  if (base.size() != 12) {
    set_last_error("cmm_mesh_create: expected 12 vertices of valence 5");
    return CMM_ERR_MESH;
  }
  // shortest edge, for the lookup grid
  double emin = 1e300;
  for (int t = 0; t < nt; ++t)
    for (int e = 0; e < 3; ++e) {
      D3 a = vtx(verts, tris[3 * t + e]), b = vtx(verts, tris[3 * t + (e + 1) % 3]);
      emin = std::min(emin, norm(a - b));
    }
  if (!(emin > 0)) {
    set_last_error("cmm_mesh_create: degenerate edge");
    return CMM_ERR_MESH;
  }
  VertexGrid grid(verts, nv, 0.5 * emin);
  const double tol = 1e-6 * emin;

  // level-0 faces from the base vertices: each base vertex's 5 nearest
  // base vertices are its icosahedron neighbours
  bool adj[12][12] = {};
  for (int i = 0; i < 12; ++i) {
    std::vector<std::pair<double, int>> d;
    for (int j = 0; j < 12; ++j)
      if (j != i) d.push_back({-dot(vtx(verts, base[i]), vtx(verts, base[j])), j});
    std::sort(d.begin(), d.end());
    for (int k = 0; k < 5; ++k) adj[i][d[k].second] = true;
  }
  std::vector<int4> faces;
  for (int i = 0; i < 12; ++i)
    for (int j = i + 1; j < 12; ++j)
      for (int k = j + 1; k < 12; ++k)
        if (adj[i][j] && adj[j][i] && adj[i][k] && adj[k][i] && adj[j][k] && adj[k][j]) {
          int a = base[i], b = base[j], c = base[k];
          if (det_cols(vtx(verts, a), vtx(verts, b), vtx(verts, c)) < 0) std::swap(b, c);
          faces.push_back(make_int4(a, b, c, 0));
        }
  if (faces.size() != 20) {
    set_last_error("cmm_mesh_create: could not rebuild the base icosahedron");
    return CMM_ERR_MESH;
  }
  // root tables
  std::vector<double> root(20 * 12);
  std::vector<int> root_adj(20 * 3, -1);
  for (int f = 0; f < 20; ++f) {
    D3 a = vtx(verts, faces[f].x), b = vtx(verts, faces[f].y), c = vtx(verts, faces[f].z);
    D3 cen = unit(a + b + c), n0 = unit(cross(a, b)), n1 = unit(cross(b, c)), n2 = unit(cross(c, a));
    double* r = &root[12 * f];
    r[0] = cen.x; r[1] = cen.y; r[2] = cen.z;
    r[3] = n0.x; r[4] = n0.y; r[5] = n0.z;
    r[6] = n1.x; r[7] = n1.y; r[8] = n1.z;
    r[9] = n2.x; r[10] = n2.y; r[11] = n2.z;
    int ev[3][2] = {{faces[f].x, faces[f].y}, {faces[f].y, faces[f].z}, {faces[f].z, faces[f].x}};
    for (int e = 0; e < 3; ++e)
      for (int g = 0; g < 20; ++g) {
        if (g == f) continue;
        int gv[3] = {faces[g].x, faces[g].y, faces[g].z};
        int hit = 0;
        for (int q = 0; q < 3; ++q) hit += (gv[q] == ev[e][0]) + (gv[q] == ev[e][1]);
        if (hit == 2) root_adj[3 * f + e] = g;
      }
  }
  // refinement hierarchy
  const int64_t nnodes = (nt_exp - 20) / 3;  // 20 (4^level - 1) / 3
  std::vector<double> node_n(9 * std::max<int64_t>(nnodes, 1));
  std::vector<float> node_nf(9 * std::max<int64_t>(nnodes, 1));
  std::vector<int4> cur = faces, next;
  std::unordered_map<int64_t, int> mids;
  int64_t off = 0;
  for (int j = 0; j < level; ++j) {
    next.resize(cur.size() * 4);
    for (size_t f = 0; f < cur.size(); ++f) {
      int a = cur[f].x, b = cur[f].y, c = cur[f].z;
      int mv[3];
      int ends[3][2] = {{a, b}, {b, c}, {c, a}};
      for (int e = 0; e < 3; ++e) {
        int u = std::min(ends[e][0], ends[e][1]), w = std::max(ends[e][0], ends[e][1]);
        int64_t k = (int64_t)u * nv + w;
        auto it = mids.find(k);
        if (it != mids.end()) {
          mv[e] = it->second;
          continue;
        }
        int id = grid.find(unit(vtx(verts, u) + vtx(verts, w)), tol);
        if (id < 0) {
          set_last_error("cmm_mesh_create: an edge midpoint is not a mesh vertex (not an icosahedral refinement)");
          return CMM_ERR_MESH;
        }
        mids[k] = id;
        mv[e] = id;
      }
      int mab = mv[0], mbc = mv[1], mca = mv[2];
      D3 pab = vtx(verts, mab), pbc = vtx(verts, mbc), pca = vtx(verts, mca);
      D3 n[3] = {unit(cross(pab, pca)), unit(cross(pbc, pab)), unit(cross(pca, pbc))};
      double* dst = &node_n[9 * (off + f)];
      float* dstf = &node_nf[9 * (off + f)];
      for (int i = 0; i < 3; ++i) {
        dst[3 * i] = n[i].x; dst[3 * i + 1] = n[i].y; dst[3 * i + 2] = n[i].z;
        dstf[3 * i] = (float)n[i].x; dstf[3 * i + 1] = (float)n[i].y; dstf[3 * i + 2] = (float)n[i].z;
      }
      next[4 * f + 0] = make_int4(a, mab, mca, 0);
      next[4 * f + 1] = make_int4(mab, b, mbc, 0);
      next[4 * f + 2] = make_int4(mca, mbc, c, 0);
      next[4 * f + 3] = make_int4(mbc, mca, mab, 0);
    }
    off += cur.size();
    cur.swap(next);
    mids.clear();
  }
  // leaves -> rows of the caller's table
  std::unordered_map<int64_t, int> rowof;
  rowof.reserve(nt * 2);
  for (int t = 0; t < nt; ++t) {
    auto ins = rowof.emplace(tri_key(tris[3 * t], tris[3 * t + 1], tris[3 * t + 2], nv), t);
    if (!ins.second) {
      set_last_error("cmm_mesh_create: duplicate triangle in table");
      return CMM_ERR_MESH;
    }
  }
  std::vector<int> leaf_row(nt);
  std::vector<char> used(nt, 0);
  for (int64_t l = 0; l < nt; ++l) {
    auto it = rowof.find(tri_key(cur[l].x, cur[l].y, cur[l].z, nv));
    if (it == rowof.end() || used[it->second]) {
      set_last_error("cmm_mesh_create: triangle table is not the refinement's triangulation");
      return CMM_ERR_MESH;
    }
    used[it->second] = 1;
    leaf_row[l] = it->second;
  }
  // per-row tables
  std::vector<double> vpad(4 * (size_t)nv);
  for (int i = 0; i < nv; ++i) {
    vpad[4 * i] = verts[3 * i];
    vpad[4 * i + 1] = verts[3 * i + 1];
    vpad[4 * i + 2] = verts[3 * i + 2];
    vpad[4 * i + 3] = 0.0;
  }
  std::vector<int4> tv(nt);
  std::vector<double> loc((size_t)nt * kLocStride), asmf((size_t)nt * kAsmStride);
  for (int t = 0; t < nt; ++t) {
    tv[t] = make_int4(tris[3 * t], tris[3 * t + 1], tris[3 * t + 2], 0);
    D3 v1 = vtx(verts, tris[3 * t]), v2 = vtx(verts, tris[3 * t + 1]), v3 = vtx(verts, tris[3 * t + 2]);
    location_record(v1, v2, v3, &loc[(size_t)t * kLocStride]);
    assembly_factors(v1, v2, v3, &asmf[(size_t)t * kAsmStride]);
  }
  // walk tables: inward edge normals and the row across each edge
  std::vector<float> walk_f((size_t)nt * kWalkStride, 0.f);
  std::vector<double> walk_d((size_t)nt * kWalkStride, 0.0);
  {
    // undirected edge -> the (at most two) rows that contain it
    std::unordered_map<int64_t, std::pair<int, int>> edge_rows;
    edge_rows.reserve((size_t)nt * 2);
    for (int t = 0; t < nt; ++t)
      for (int e = 0; e < 3; ++e) {
        const int u = tris[3 * t + e], w = tris[3 * t + (e + 1) % 3];
        auto ins = edge_rows.emplace((int64_t)std::min(u, w) * nv + std::max(u, w), std::make_pair(t, -1));
        if (!ins.second) {
          if (ins.first->second.second >= 0) {
            set_last_error("cmm_mesh_create: an edge is shared by more than two triangles");
            return CMM_ERR_MESH;
          }
          ins.first->second.second = t;
        }
      }
    for (int t = 0; t < nt; ++t) {
      const int a[3] = {tris[3 * t], tris[3 * t + 1], tris[3 * t + 2]};
      const double det = det_cols(vtx(verts, a[0]), vtx(verts, a[1]), vtx(verts, a[2]));
      const double sgn = det < 0 ? -1.0 : 1.0;
      // barycentric b_i = R_i . q = s_i (n . q) with n the inward unit
      // normal of the edge opposite vertex i (edge (i+1, i+2)) and
      // s_i = |v_{i+1} x v_{i+2}| / |det| > 0, stored in floats 12..14
      for (int i = 0; i < 3; ++i)
        walk_f[(size_t)t * kWalkStride + 12 + i] =
            (float)(norm(cross(vtx(verts, a[(i + 1) % 3]), vtx(verts, a[(i + 2) % 3]))) / std::fabs(det));
      for (int e = 0; e < 3; ++e) {
        const int u = a[e], w = a[(e + 1) % 3];
        // the same plane seen from the row across the edge has exactly the
        // negated normal (cross(w, u) = -cross(u, w) in FP64 without
        // contraction), so the two rows' side decisions never conflict
        const D3 n = sgn * unit(cross(vtx(verts, u), vtx(verts, w)));
        const auto& pr = edge_rows[(int64_t)std::min(u, w) * nv + std::max(u, w)];
        const int nb = pr.first == t ? pr.second : pr.first;
        if (nb < 0) {
          set_last_error("cmm_mesh_create: an edge has no second triangle (not a closed triangulation)");
          return CMM_ERR_MESH;
        }
        float* f = &walk_f[(size_t)t * kWalkStride + 4 * e];
        f[0] = (float)n.x;
        f[1] = (float)n.y;
        f[2] = (float)n.z;
        std::memcpy(&f[3], &nb, sizeof(int));
        double* d = &walk_d[(size_t)t * kWalkStride + 3 * e];
        d[0] = n.x;
        d[1] = n.y;
        d[2] = n.z;
      }
    }
  }
  hm->walk_f.swap(walk_f);
  hm->walk_d.swap(walk_d);
  hm->level = level;
  hm->nv = nv;
  hm->nt = nt;
  hm->vpad.swap(vpad);
  hm->tv.swap(tv);
  hm->loc.swap(loc);
  hm->asmf.swap(asmf);
  hm->root.swap(root);
  hm->root_adj.swap(root_adj);
  hm->node_n.swap(node_n);
  hm->node_nf.swap(node_nf);
  hm->leaf_row.swap(leaf_row);
  return CMM_OK;
}

int upload_asm_factors(DeviceBuffer& dst, const std::vector<double>& asmf, int nt) {
  std::vector<double> soa((size_t)kAsmFactors * nt);
  for (int t = 0; t < nt; ++t)
    for (int j = 0; j < kAsmFactors; ++j) soa[(size_t)j * nt + t] = asmf[(size_t)t * kAsmStride + j];
  return dst.upload(soa.data(), soa.size() * 8);
}

int upload_mesh(const HostMesh& h, cmm_mesh* m) {
  const int level = h.level, nv = h.nv, nt = h.nt;
  int rc;
  if ((rc = m->verts.upload(h.vpad.data(), h.vpad.size() * 8))) return rc;
  if ((rc = m->tri_v.upload(h.tv.data(), h.tv.size() * sizeof(int4)))) return rc;
  if ((rc = m->tri_loc.upload(h.loc.data(), h.loc.size() * 8))) return rc;
  if ((rc = upload_asm_factors(m->tri_asm, h.asmf, nt))) return rc;
  if ((rc = m->root.upload(h.root.data(), h.root.size() * 8))) return rc;
  {
    std::vector<float> rf(h.root.begin(), h.root.end());
    if ((rc = m->root_f.upload(rf.data(), rf.size() * 4))) return rc;
  }
  if ((rc = m->root_adj.upload(h.root_adj.data(), h.root_adj.size() * 4))) return rc;
  if ((rc = m->node_n.upload(h.node_n.data(), h.node_n.size() * 8))) return rc;
  if ((rc = m->node_nf.upload(h.node_nf.data(), h.node_nf.size() * 4))) return rc;
  if ((rc = m->leaf_row.upload(h.leaf_row.data(), h.leaf_row.size() * 4))) return rc;
  if ((rc = m->walk_f.upload(h.walk_f.data(), h.walk_f.size() * 4))) return rc;
  if ((rc = m->walk_d.upload(h.walk_d.data(), h.walk_d.size() * 8))) return rc;
  int zero = 0;
  if ((rc = m->status.upload(&zero, sizeof(int)))) return rc;
  MeshView& v = m->view;
  v.level = level;
  v.nv = nv;
  v.nt = nt;
  v.verts = (const double*)m->verts.p;
  v.tri_v = (const int4*)m->tri_v.p;
  v.tri_loc = (const double*)m->tri_loc.p;
  v.tri_asm = (const double*)m->tri_asm.p;
  v.root = (const double*)m->root.p;
  v.root_f = (const float*)m->root_f.p;
  v.root_adj = (const int*)m->root_adj.p;
  v.node_n = (const double*)m->node_n.p;
  v.node_nf = (const float*)m->node_nf.p;
  v.leaf_row = (const int*)m->leaf_row.p;
  v.walk_f = (const float*)m->walk_f.p;
  v.walk_d = (const double*)m->walk_d.p;
  v.jump = nullptr;
  v.status = (int*)m->status.p;
  return build_jump_table(m);
}

}  // namespace cmm
