"""Icosahedral and MWSS lat-lon mesh builders (host side, numpy).

The reference loads pickled icosahedral meshes produced by stripy
(``cmm_s2/tests/precompute_meshes.py:13-17``) and builds the lat-lon
velocity mesh from the MWSS sample positions
(``cmm_s2/core/mesh_functions.py:175-194``).  Neither the pickles nor stripy
are available, so the vertex sets are generated here:

* ``icosahedral_mesh(level)``: the regular icosahedron with its two poles on
  the z axis, refined ``level`` times by normalised edge-midpoint bisection.
  Vertex 0 is the north pole and the last vertex is the south pole, which is
  what ``spherical_triangulation.stencil_pts`` assumes when it patches the
  tangent frames of the first and last vertices
  (``cmm_s2/core/mesh_functions.py:137-142``).
  Triangles are returned in hierarchical order: triangle ``4*f + c`` at level
  ``j+1`` is child ``c`` of triangle ``f`` at level ``j``.
* ``mwss_angles(L)``: MWSS colatitudes ``pi*t/L`` (t = 0..L) and longitudes
  ``2*pi*p/(2L)`` (p = 0..2L-1), the ``pyssht.sample_positions(L, "MWSS")``
  convention the reference relies on.
"""
import numpy as np


def _base_icosahedron():
    z = np.arctan(0.5)
    pts = [(0.0, 0.0, 1.0)]
    for k in range(5):
        lon = 2 * np.pi * k / 5
        pts.append((np.cos(z) * np.cos(lon), np.cos(z) * np.sin(lon), np.sin(z)))
    for k in range(5):
        lon = 2 * np.pi * k / 5 + np.pi / 5
        pts.append((np.cos(z) * np.cos(lon), np.cos(z) * np.sin(lon), -np.sin(z)))
    pts.append((0.0, 0.0, -1.0))
    faces = []
    for k in range(5):
        u0, u1 = 1 + k, 1 + (k + 1) % 5
        l0, l1 = 6 + k, 6 + (k + 1) % 5
        faces.append((0, u0, u1))
        faces.append((u0, l0, u1))
        faces.append((u1, l0, l1))
        faces.append((l0, 11, l1))
    return np.array(pts, dtype=np.float64), np.array(faces, dtype=np.int64)


def _orient_ccw(verts, faces):
    a, b, c = verts[faces[:, 0]], verts[faces[:, 1]], verts[faces[:, 2]]
    d = np.einsum("ij,ij->i", a, np.cross(b, c))
    flip = d < 0
    faces = faces.copy()
    faces[flip, 1], faces[flip, 2] = faces[flip, 2].copy(), faces[flip, 1].copy()
    return faces


def icosahedral_mesh(level):
    """Return ``(verts (Nv,3) float64, tris (Nt,3) int32)`` for a level-``level``
    icosahedral refinement; Nv = 10*4**level + 2, Nt = 20*4**level.

    Children of a counter-clockwise face (a, b, c) with normalised edge
    midpoints mab, mbc, mca are, in order:
    (a, mab, mca), (mab, b, mbc), (mca, mbc, c), (mbc, mca, mab).
    """
    verts, faces = _base_icosahedron()
    faces = _orient_ccw(verts, faces)
    for _ in range(level):
        nv = len(verts)
        a, b, c = faces[:, 0], faces[:, 1], faces[:, 2]
        edges = np.concatenate([np.stack([a, b], 1), np.stack([b, c], 1), np.stack([c, a], 1)])
        key = np.minimum(edges[:, 0], edges[:, 1]) * nv + np.maximum(edges[:, 0], edges[:, 1])
        ukey, inv = np.unique(key, return_inverse=True)
        e0, e1 = ukey // nv, ukey % nv
        mid = verts[e0] + verts[e1]
        mid /= np.linalg.norm(mid, axis=1)[:, None]
        mid_id = nv + np.arange(len(ukey))
        nf = len(faces)
        mab, mbc, mca = mid_id[inv[:nf]], mid_id[inv[nf:2 * nf]], mid_id[inv[2 * nf:]]
        children = np.stack([
            np.stack([a, mab, mca], 1),
            np.stack([mab, b, mbc], 1),
            np.stack([mca, mbc, c], 1),
            np.stack([mbc, mca, mab], 1)], 1)
        faces = children.reshape(-1, 3)
        verts = np.concatenate([verts, mid])
    # move the south pole (base vertex 11) to the end
    nv = len(verts)
    order = np.concatenate([np.arange(11), np.arange(12, nv), [11]])
    remap = np.empty(nv, dtype=np.int64)
    remap[order] = np.arange(nv)
    verts = np.ascontiguousarray(verts[order])
    faces = remap[faces]
    return verts, faces.astype(np.int32)


def mwss_angles(L):
    """MWSS colatitudes (L+1,) and longitudes (2L,)."""
    return np.pi * np.arange(L + 1) / L, 2 * np.pi * np.arange(2 * L) / (2 * L)


def latlon_mesh_arrays(L):
    """Arrays of the MWSS lat-lon velocity mesh as the reference builds them
    (cmm_s2/core/mesh_functions.py:175-194, 332-350): ring colatitudes
    theta (L+1,), longitudes phi (2L,), ring points grid (3, L+1, 2L) =
    sphere2cart(phi, theta), and the mesh vertices (2+(L-1)*2L, 3): north
    pole, interior rings row by row, south pole, converted from
    (lon, lat = pi/2 - theta) the way stripy does."""
    theta, phi = mwss_angles(L)
    Phi, The = np.meshgrid(phi, theta)
    grid = np.array([np.sin(The) * np.cos(Phi), np.sin(The) * np.sin(Phi), np.cos(The)])
    XX = np.meshgrid(phi, theta[1:-1])
    lons = np.concatenate([[0.0], XX[0].reshape(-1), [0.0]])
    lats = np.concatenate([[np.pi / 2], -XX[1].reshape(-1) + np.pi / 2, [-np.pi / 2]])
    verts = np.stack([np.cos(lats) * np.cos(lons), np.cos(lats) * np.sin(lons), np.sin(lats)], 1)
    return theta, phi, grid, verts


def _cross(a, b):
    return np.stack([a[:, 1] * b[:, 2] - a[:, 2] * b[:, 1], a[:, 2] * b[:, 0] - a[:, 0] * b[:, 2],
                     a[:, 0] * b[:, 1] - a[:, 1] * b[:, 0]], 1)


def _unit(x):
    n = np.sqrt(x[:, 0] ** 2 + x[:, 1] ** 2 + x[:, 2] ** 2)
    return np.stack([x[:, 0] / n, x[:, 1] / n, x[:, 2] / n], 1)


def stencil_frames(verts, eps=1e-5):
    """Per-vertex tangent frames (2,Nv,3) and the four stencil points
    (3,4,Nv) at distance eps (spherical_triangulation.stencil_pts,
    cmm_s2/core/mesh_functions.py:128-166): a1 = v x e_z, a2 = v x a1
    (first and last vertex, the poles, use fixed directions), stencil
    points v -+ eps a1 -+ eps a2 lifted back onto the sphere along v."""
    ez = np.broadcast_to([0.0, 0.0, 1.0], verts.shape)
    a1 = _cross(verts, ez)
    a2 = _cross(verts, a1)
    s = 1 / np.sqrt(2)
    a1[0] = _cross(verts[:1], np.array([[s, 0.0, s]]))[0]
    a1[-1] = _cross(verts[-1:], np.array([[s, 0.0, -s]]))[0]
    a2[0] = _cross(verts[:1], a1[:1])[0]
    a2[-1] = _cross(verts[-1:], a1[-1:])[0]
    a1n, a2n = _unit(a1), _unit(a2)
    pts = []
    for sa, sb in ((-1, -1), (1, -1), (-1, 1), (1, 1)):
        y = verts + sa * a1n * eps + sb * a2n * eps
        yn = y[:, 0] * verts[:, 0] + y[:, 1] * verts[:, 1] + y[:, 2] * verts[:, 2]
        tt = -yn + np.sqrt(yn ** 2 - (y[:, 0] ** 2 + y[:, 1] ** 2 + y[:, 2] ** 2) + 1)
        pts.append(y + tt[:, None] * verts)
    s_pts = np.stack([np.stack([p[:, c] for p in pts]) for c in range(3)])
    return np.stack([a1n, a2n]), s_pts


def identity_jets(verts):
    """Jets (3,4,Nv) of the identity map: value x_c, gradient of x_c the
    tangent projection of e_c (cmm_s2/core/spherical_simulations.py:165-169)."""
    x = verts.T
    jets = np.zeros((3, 4, len(verts)))
    jets[:, 0] = x
    P = np.eye(3)[:, :, None] - x[:, None, :] * x[None, :, :]
    for k in range(3):
        jets[k, 1:] = P[:, k]
    return jets


def random_sphere_points(n, seed):
    """``n`` points uniform on the unit sphere (normalised Gaussians), (n,3)."""
    rng = np.random.default_rng(seed)
    x = rng.standard_normal((n, 3))
    return x / np.linalg.norm(x, axis=1)[:, None]
