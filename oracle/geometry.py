"""Geometry, point location and mesh tables (oracle restatement).

Each function names the reference code it restates (paths relative to the
reference repository).  Arrays use the reference's conventions: points are
(N,3) unless a docstring says (3,N).
"""
import numpy as np
from scipy.spatial import cKDTree


# ---------------------------------------------------------------- utils.py
def sphere2cart(phi, theta):
    """cmm_s2/core/utils.py:9-13."""
    return [np.sin(theta) * np.cos(phi), np.sin(theta) * np.sin(phi), np.cos(theta)]


def cart2sphere(xyz):
    """cmm_s2/core/utils.py:18-23; xyz indexed by component first, phi in [0, 2pi)."""
    x, y, z = xyz[0], xyz[1], xyz[2]
    return [(np.arctan2(y, x) + 2 * np.pi) % (2 * np.pi), np.arctan2(np.sqrt(y ** 2 + x ** 2), z)]


def det_cols(a, b, c):
    """Determinant of the 3x3 matrix with columns a, b, c (each (N,3)).

    Same six-term expansion and term order as cmm_s2/core/utils.py:49-56."""
    return (a[:, 0] * b[:, 1] * c[:, 2] + b[:, 0] * c[:, 1] * a[:, 2] + a[:, 1] * b[:, 2] * c[:, 0]
            - (c[:, 0] * b[:, 1] * a[:, 2] + c[:, 1] * b[:, 2] * a[:, 0] + b[:, 0] * a[:, 1] * c[:, 2]))


def bary(v1, v2, v3, q):
    """Un-normalised spherical barycentric coordinates, cmm_s2/core/utils.py:58-67."""
    d = det_cols(v1, v2, v3)
    return np.stack([det_cols(q, v2, v3) / d, det_cols(v1, q, v3) / d, det_cols(v1, v2, q) / d], axis=1)


def unit_rows(x):
    """Row normalisation (utils.div_norm, cmm_s2/core/utils.py:36-38), returns (N,3)."""
    n = np.sqrt(x[:, 0] ** 2 + x[:, 1] ** 2 + x[:, 2] ** 2)
    return np.stack([x[:, 0] / n, x[:, 1] / n, x[:, 2] / n], axis=1)


def cross_rows(a, b):
    return np.stack([a[:, 1] * b[:, 2] - a[:, 2] * b[:, 1],
                     a[:, 2] * b[:, 0] - a[:, 0] * b[:, 2],
                     a[:, 0] * b[:, 1] - a[:, 1] * b[:, 0]], axis=1)


def dot_rows(a, b):
    return a[:, 0] * b[:, 0] + a[:, 1] * b[:, 1] + a[:, 2] * b[:, 2]


def tan_unit(a, b):
    """Unit tangent projection of a at the unit point b: mesh_functions.sphere_tan_proj
    (cmm_s2/core/mesh_functions.py:320-329)."""
    c = dot_rows(b, a)
    d = np.sqrt(dot_rows(a, a) - 2 * c ** 2 + dot_rows(b, b) * c ** 2)
    return np.stack([(a[:, 0] - c * b[:, 0]) / d, (a[:, 1] - c * b[:, 1]) / d,
                     (a[:, 2] - c * b[:, 2]) / d], axis=1)


# ------------------------------------------------------- Powell-Sabin split
def ps_split(verts, tris):
    """Per-triangle Powell-Sabin geometry (cmm_s2/core/mesh_functions.py:92-126).

    Returns H (9,Nt,3): unit tangents h12,h21,h23,h32,h13,h31,h41,h42,h43;
    G (10,Nt,3): barycentrics g12,g21,g23,g32,g13,g31,g14,g24,g34,mid;
    E (3,Nt,3): barycentrics of the edge midpoints e1,e2,e3 in (v1,v2,v3)."""
    v1, v2, v3 = verts[tris[:, 0]], verts[tris[:, 1]], verts[tris[:, 2]]
    v4 = unit_rows((v1 + v2 + v3) / 3)
    e1, e2, e3 = unit_rows(v1 / 2 + v2 / 2), unit_rows(v2 / 2 + v3 / 2), unit_rows(v3 / 2 + v1 / 2)
    h12, h21, h23 = tan_unit(v2 - v1, v1), tan_unit(v1 - v2, v2), tan_unit(v3 - v2, v2)
    h32, h13, h31 = tan_unit(v2 - v3, v3), tan_unit(v3 - v1, v1), tan_unit(v1 - v3, v3)
    h41, h42, h43 = tan_unit(v4 - v1, v1), tan_unit(v4 - v2, v2), tan_unit(v4 - v3, v3)
    g12, g21 = bary(v1, e1, v4, h12), bary(v2, v4, e1, h21)
    g23, g32 = bary(v2, e2, v4, h23), bary(v3, v4, e2, h32)
    g13, g31 = bary(v1, v4, e3, h13), bary(v3, e3, v4, h31)
    g14 = bary(v1, v4, e3, tan_unit(v4, v1))
    g24 = bary(v2, v4, e1, tan_unit(v4, v2))
    g34 = bary(v3, v4, e2, tan_unit(v4, v3))
    mid = bary(v1, v2, v3, v4)
    E = np.stack([bary(v1, v2, v3, e1), bary(v1, v2, v3, e2), bary(v1, v2, v3, e3)])
    H = np.stack([h12, h21, h23, h32, h13, h31, h41, h42, h43])
    G = np.stack([g12, g21, g23, g32, g13, g31, g14, g24, g34, mid])
    return H, G, E


def stencil_points(verts, eps=1e-5):
    """Vertex tangent frames and the 4 stencil points per vertex
    (cmm_s2/core/mesh_functions.py:128-166).

    Returns tan (2,Nv,3) = (a1_n, a2_n) and s_pts (3,4,Nv)."""
    a1 = cross_rows(verts, np.broadcast_to([0.0, 0.0, 1.0], verts.shape))
    a2 = cross_rows(verts, a1)
    s = 1 / np.sqrt(2)
    a1[0] = cross_rows(verts[:1], np.array([[s, 0.0, s]]))[0]
    a1[-1] = cross_rows(verts[-1:], np.array([[s, 0.0, -s]]))[0]
    a2[0] = cross_rows(verts[:1], a1[:1])[0]
    a2[-1] = cross_rows(verts[-1:], a1[-1:])[0]
    a1n, a2n = unit_rows(a1), unit_rows(a2)

    def lift(y, n):  # utils.pi_proj, cmm_s2/core/utils.py:136-139
        yn = dot_rows(y, n)
        tt = -yn + np.sqrt(yn ** 2 - dot_rows(y, y) + 1)
        return y + tt[:, None] * n

    pts = [lift(verts - a1n * eps - a2n * eps, verts), lift(verts + a1n * eps - a2n * eps, verts),
           lift(verts - a1n * eps + a2n * eps, verts), lift(verts + a1n * eps + a2n * eps, verts)]
    s_pts = np.stack([np.stack([p[:, c] for p in pts]) for c in range(3)])
    return np.stack([a1n, a2n]), s_pts


# ----------------------------------------------------------- point location
class ConeLocator:
    """Containing spherical triangle by cone tests on candidate triangles.

    The reference locates with Qhull's ``find_simplex`` on the tetrahedra
    (origin, triangle) of the ball (cmm_s2/core/mesh_functions.py:43, 82):
    q/2 lies in a tetrahedron exactly when q lies in the cone of its
    triangle.  This restates that predicate directly: a query belongs to a
    counter-clockwise triangle (a,b,c) when det(a,b,q), det(b,c,q) and
    det(c,a,q) are all >= 0.  Candidates are the triangles with the nearest
    centroids; queries none of them contains fall back to a full scan.
    Points on a shared edge are legitimately claimed by either triangle."""

    def __init__(self, verts, tris, k=8):
        self.verts, self.tris = verts, tris
        a, b, c = verts[tris[:, 0]], verts[tris[:, 1]], verts[tris[:, 2]]
        self.n = np.stack([cross_rows(a, b), cross_rows(b, c), cross_rows(c, a)], 1)  # (Nt,3,3)
        self.tree = cKDTree(unit_rows(a + b + c))
        self.k = min(k, len(tris))

    def locate(self, q):
        """Triangle ids (N,); -1 for non-finite queries (as find_simplex)."""
        fin = np.isfinite(q).all(axis=1)
        if not fin.all():
            tri = np.full(len(q), -1, dtype=np.int64)
            tri[fin] = self.locate(q[fin])
            return tri
        _, cand = self.tree.query(q, k=self.k)
        cand = cand.reshape(len(q), -1)
        tri = np.full(len(q), -1, dtype=np.int64)
        for j in range(cand.shape[1]):
            todo = tri < 0
            if not todo.any():
                break
            c = cand[todo, j]
            s = np.einsum("nij,nj->ni", self.n[c], q[todo])
            ok = (s >= 0).all(axis=1)
            idx = np.nonzero(todo)[0][ok]
            tri[idx] = c[ok]
        for i in np.nonzero(tri < 0)[0]:
            s = self.n @ q[i]
            tri[i] = int(np.argmax(s.min(axis=1)))
        return tri


class QhullLocator:
    """The reference's own locator: scipy ``Delaunay`` of {origin} and the
    vertices, ``find_simplex(q/2)`` (cmm_s2/core/mesh_functions.py:41-56, 82).

    ``tris`` is the orientation-fixed simplex table in Qhull order."""

    def __init__(self, verts):
        from scipy.spatial import Delaunay
        self.d = Delaunay(np.vstack([np.zeros(3), verts]))
        simp = self.d.simplices - 1
        tris = np.array([t[t != -1] for t in simp])
        v = verts[tris]
        flip = det_cols(v[:, 0], v[:, 1], v[:, 2]) < 0
        tris[flip, 1], tris[flip, 2] = tris[flip, 2].copy(), tris[flip, 1].copy()
        self.tris = tris

    def locate(self, q):
        return self.d.find_simplex(q / 2)


def query(verts, tris, locator, q):
    """spherical_triangulation.query (cmm_s2/core/mesh_functions.py:68-88):
    returns bcc (N,3), tri (N,), vs (N,3,3)."""
    tri = locator.locate(q)
    vs = verts[tris[tri]]
    return bary(vs[:, 0], vs[:, 1], vs[:, 2], q), tri, vs


def edge_distance(verts, tris, tri, q):
    """Smallest |n_e . q| over the three edge great circles of ``tri``, with
    n_e the unit normal of the edge's plane; used to classify near-edge
    queries for the location-parity rule."""
    v = verts[tris[tri]]
    d = np.full(len(q), np.inf)
    for i, j in ((0, 1), (1, 2), (2, 0)):
        n = cross_rows(v[:, i], v[:, j])
        n /= np.linalg.norm(n, axis=1)[:, None]
        d = np.minimum(d, np.abs(dot_rows(n, q)))
    return d


# ------------------------------------------------- MWSS lat-lon velocity mesh
class LatLonMesh:
    """structure_spherical_triangulation (cmm_s2/core/mesh_functions.py:169-318).

    Vertices: north pole, the L-1 interior MWSS rings of 2L points each
    (row-major), south pole.  Vertex coordinates follow stripy's lon/lat to
    Cartesian conversion with lat = pi/2 - theta
    (cmm_s2/core/mesh_functions.py:332-350)."""

    def __init__(self, L):
        self.L = L
        self.theta = np.pi * np.arange(L + 1) / L
        self.phi = 2 * np.pi * np.arange(2 * L) / (2 * L)
        N, M = 2 * L, L + 1
        Phi, The = np.meshgrid(self.phi, self.theta)
        self.grid_points = sphere2cart(Phi, The)
        lons = list(np.meshgrid(self.phi, self.theta[1:-1])[0].reshape(N * (M - 2)))
        lats = list(-np.meshgrid(self.phi, self.theta[1:-1])[1].reshape(N * (M - 2)) + np.pi / 2)
        lons = np.array([0.0] + lons + [0.0])
        lats = np.array([np.pi / 2] + lats + [-np.pi / 2])
        self.vertices = np.stack([np.cos(lats) * np.cos(lons), np.cos(lats) * np.sin(lons), np.sin(lats)], 1)
        self.simplices, self.msimplices = self._assemble(N, M)

    @staticmethod
    def _assemble(N, M):
        """grid_assemble + full_assembly (cmm_s2/core/mesh_functions.py:352-412)."""
        tris = [[0, i + 1, i + 2] for i in range(N - 1)] + [[0, N, 1]]
        for i in range(M - 3):
            for j in range(1, N + 1):
                k = j + i * N
                if j != N:
                    tris += [[k, k + N + 1, k + 1], [k, k + N, k + N + 1]]
                else:
                    tris += [[k, k + 1, i * N + 1], [k, k + N, k + 1]]
        nn = (M - 3) * N + 1
        tris += [[i, nn + N, i + 1] for i in range(nn, nn + N - 1)]
        tris += [[nn + N - 1, nn + N, nn]]
        tris = np.array(tris, dtype=np.int64)
        nt = len(tris)
        ms = np.empty((M - 1, N, 2), dtype=np.int64)
        ms[0, :, 0] = ms[0, :, 1] = np.arange(N)
        k = N
        for i in range(1, M - 2):
            ms[i, :, 0] = k + 2 * np.arange(N)
            ms[i, :, 1] = k + 2 * np.arange(N) + 1
            k += 2 * N
        ms[M - 2, :, 0] = ms[M - 2, :, 1] = nt - N + np.arange(N)
        return tris, ms

    def cells(self, q):
        """inds (cmm_s2/core/mesh_functions.py:201-255): (phi_l, theta_l)."""
        phiq, thetaq = cart2sphere(q.T)
        N, M = len(self.phi), len(self.theta)
        dphi = abs(self.phi[1] - self.phi[0])
        dthe = abs(self.theta[1] - self.theta[0])
        phiq_n = phiq % (2 * np.pi)
        phi_l = ((phiq_n - self.phi[0]) // dphi).astype(int) % N
        theta_l = ((thetaq - self.theta[0]) // dthe).astype(int)
        theta_l[theta_l == M - 1] = M - 2
        theta_c = (thetaq - self.theta[theta_l]) / dthe
        i0 = np.nonzero((theta_c <= 0.03) & (theta_l != 0))[0]
        i1 = np.nonzero((theta_c > 0.85) & (theta_l != M - 2))[0]
        phi_p1 = (phi_l + 1) % N
        the_p1 = theta_l + 1
        if len(i0):
            a = np.array(sphere2cart(self.phi[phi_l[i0]], self.theta[theta_l[i0]])).T
            b = np.array(sphere2cart(self.phi[phi_p1[i0]], self.theta[theta_l[i0]])).T
            qq = np.array(sphere2cart(phiq_n[i0], thetaq[i0])).T
            s0 = np.heaviside(dot_rows(cross_rows(a, b), qq), 0).astype(int)
        if len(i1):
            a = np.array(sphere2cart(self.phi[phi_l[i1]], self.theta[the_p1[i1]])).T
            b = np.array(sphere2cart(self.phi[phi_p1[i1]], self.theta[the_p1[i1]])).T
            qq = np.array(sphere2cart(phiq_n[i1], thetaq[i1])).T
            s1 = np.heaviside(-dot_rows(cross_rows(a, b), qq), 0).astype(int)
        if len(i0):
            theta_l[i0] -= s0
        if len(i1):
            theta_l[i1] += s1
        return phi_l, theta_l

    def query(self, q):
        """containing_simplex_and_bcc_structured
        (cmm_s2/core/mesh_functions.py:257-282): bcc (N,3), tri (N,), vs (N,3,3)."""
        phi_l, theta_l = self.cells(q)
        N = len(self.phi)
        a = np.array(sphere2cart(self.phi[phi_l], self.theta[theta_l])).T
        b = np.array(sphere2cart(self.phi[(phi_l + 1) % N], self.theta[theta_l + 1])).T
        s = np.heaviside(-dot_rows(cross_rows(a, b), q), 0).astype(int)
        tri = self.msimplices[theta_l, phi_l, s]
        vs = self.vertices[self.simplices[tri]]
        return bary(vs[:, 0], vs[:, 1], vs[:, 2], q), tri, vs
