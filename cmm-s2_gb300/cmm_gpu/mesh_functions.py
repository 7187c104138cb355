"""Meshes with the interface of cmm_s2/core/mesh_functions.py, backed by
libcmmgpu.so.

Arrays returned by queries are CUDA tensors (float64 / int32); inputs may be
numpy arrays or tensors.  Set-up tables (vertices, triangle table, tangent
frames, stencil points) stay numpy arrays on the host, as in the
reference, with device copies alongside.
"""
import numpy as np
import torch

from . import native
from .meshgen import latlon_mesh_arrays, stencil_frames


def as_device(a, device=None, dtype=torch.float64):
    if isinstance(a, torch.Tensor):
        return a.to(device=device or a.device, dtype=dtype).contiguous()
    dev = device or torch.device("cuda", torch.cuda.current_device())
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64 if dtype == torch.float64 else None)).to(dev)


def _level_of(nv):
    k, n = 0, 12
    while n < nv:
        k += 1
        n = 10 * 4 ** k + 2
    if n != nv:
        raise ValueError(f"{nv} vertices is not an icosahedral refinement")
    return k


class spherical_triangulation:
    """Icosahedral mesh (spherical_triangulation,
    cmm_s2/core/mesh_functions.py:15-166).

    pts (N,3): the vertices; simplices (Nt,3): the triangle table whose row
    indices queries report -- pass the reference mesh's ``simplices`` for
    index parity with it.  Without a table, the convex hull's facets are
    used (the same triangle set as the reference's Delaunay table, in
    another order)."""

    def __init__(self, pts, simplices=None, device=None):
        self.vertices = np.ascontiguousarray(pts, dtype=np.float64)
        if simplices is None:
            from scipy.spatial import ConvexHull
            simplices = ConvexHull(self.vertices).simplices
            v = self.vertices[simplices]
            flip = np.einsum("ij,ij->i", v[:, 0], np.cross(v[:, 1], v[:, 2])) < 0
            simplices[flip, 1], simplices[flip, 2] = simplices[flip, 2].copy(), simplices[flip, 1].copy()
        self.simplices = np.ascontiguousarray(simplices, dtype=np.int32)
        self.x, self.y, self.z = self.vertices[:, 0], self.vertices[:, 1], self.vertices[:, 2]
        self.level = _level_of(len(self.vertices))
        self.native = native.Mesh(self.vertices, self.simplices, self.level, device=device)
        self.device = self.native.device
        tan, s_pts = stencil_frames(self.vertices)
        self.tan_vects = [tan[0], tan[1]]
        self.s_pts = s_pts
        self.tan_d = torch.from_numpy(np.ascontiguousarray(tan)).to(self.device)
        self.s_pts_d = torch.from_numpy(np.ascontiguousarray(s_pts)).to(self.device)

    @classmethod
    def from_reference(cls, mesh, device=None):
        return cls(np.asarray(mesh.vertices), np.asarray(mesh.simplices), device)

    def query(self, q_pts):
        """(bcc (N,3), trangs (N,), vs (N,3,3)) (mesh_functions.py:68-88)."""
        q = as_device(q_pts, self.device)
        tri, bcc = self.native.locate(q)
        v = torch.from_numpy(self.vertices).to(self.device)
        s = torch.from_numpy(self.simplices.astype(np.int64)).to(self.device)
        return bcc, tri, v[s[tri.long()]]


class structure_spherical_triangulation:
    """MWSS lat-lon velocity mesh (mesh_functions.py:169-318)."""

    def __init__(self, L, device=None):
        theta, phi, grid, verts = latlon_mesh_arrays(L)
        self.L, self.theta, self.phi = L, theta, phi
        self.grid_points = [grid[0], grid[1], grid[2]]
        self.vertices = verts
        self.native = native.VelMesh(L, theta, phi, grid, verts, device=device)
        self.device = self.native.device

    def query(self, q_pts):
        q = as_device(q_pts, self.device)
        tri, bcc = self.native.locate(q)
        return bcc, tri, None
