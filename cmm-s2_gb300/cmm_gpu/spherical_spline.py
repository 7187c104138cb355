"""Spline maps with the interface of cmm_s2/core/spherical_spline.py,
backed by libcmmgpu.so.  ``vals`` are jets (3,4,Nv) in the reference's
layout; coefficients live in the library's per-triangle records."""
import numpy as np
import torch

from . import native
from .mesh_functions import as_device


class sphere_diffeomorphism:
    """Powell-Sabin spline map (spherical_spline.py:155-337)."""

    def __init__(self, mesh, vals, coeffs=None):
        self.mesh = mesh
        self.vals = as_device(vals, mesh.device)
        self.coeffs = mesh.native.new_coeffs() if coeffs is None else coeffs
        self.assemble_coefficients(self.coeffs)

    def assemble_coefficients(self, coeffs):
        """Overwrites ``coeffs`` in place, as the reference does (:300-337)."""
        self.mesh.native.assemble(self.vals, out=coeffs)
        return coeffs

    def __call__(self, q_pts):
        """Normalised image of q_pts (N,3) -> (3,N) (:178-205)."""
        out, _, _, _ = self.mesh.native.compose([self.coeffs], as_device(q_pts, self.mesh.device))
        return out.T

    def eval_grad(self, q_pts):
        """Tangent Jacobians (N,3,3) at q_pts (the working form of :208-265)."""
        _, _, _, jac = self.mesh.native.compose([self.coeffs], as_device(q_pts, self.mesh.device),
                                                want_jac=True)
        return jac

    def stencil_eval(self, q_pts, st_pts):
        """Locate at q_pts (3,N); evaluate st_pts (3,4,N) there, un-normalised (:268-298)."""
        return self.mesh.native.stencil_eval(self.coeffs, as_device(q_pts, self.mesh.device),
                                             as_device(st_pts, self.mesh.device))


class composite_sphere_diffeomorphism:
    """Stack of submaps (spherical_spline.py:340-508)."""

    def __init__(self, mesh, vals, coeffs=None, ns=None):
        self.mesh = mesh
        n = len(vals) if vals is not None else len(ns)
        self.vals = [as_device(v, mesh.device) for v in vals] if vals is not None else [None] * n
        self.coeffs = coeffs if coeffs is not None else [mesh.native.new_coeffs() for _ in range(n)]
        self.ns = ns
        self.Nc = 0

    def assemble_coefficients(self, i, vals):
        self.vals[i] = as_device(vals, self.mesh.device).clone()
        self.mesh.native.assemble(self.vals[i], out=self.coeffs[i])

    def __call__(self, q_pts, N_c=None):
        """Apply submaps N_c-1, ..., 0 to q_pts (N,3) -> (N,3) (:365-398)."""
        n_c = self.Nc if N_c is None else N_c
        q = as_device(q_pts, self.mesh.device)
        if n_c == 0:
            return q.clone()
        out, _, _, _ = self.mesh.native.compose(self.coeffs[:n_c], q)
        return out

    def jacobian(self, q_pts, N_c=None):
        n_c = self.Nc if N_c is None else N_c
        return self.mesh.native.compose(self.coeffs[:n_c], as_device(q_pts, self.mesh.device),
                                        want_jac=True)[3]


class spline_interp_velocity:
    """Velocity interpolant with up to 3 time levels (spherical_spline.py:545-655)."""

    def __init__(self, mesh, vals, coeffs=None, ts=(0.0, 0.0, 0.0)):
        self.mesh = mesh
        self.vals = as_device(vals, mesh.device) if vals is not None else \
            torch.zeros((3, 3, 4, mesh.native.nv), dtype=torch.float64, device=mesh.device)
        self.coeffs = coeffs if coeffs is not None else [mesh.native.new_coeffs() for _ in range(3)]
        self.ts = np.asarray(ts, dtype=np.float64)
        self.stepping = False
        self.nVs = 1

    def init_coeffs(self, i):
        self.mesh.native.assemble(self.vals[i], out=self.coeffs[i])

    def __call__(self, t, dt, q_pts):
        """Velocity at q_pts (3,N) -> (3,N) (:570-615)."""
        return self.mesh.native.velocity(self.coeffs[:self.nVs], float(self.ts[0]), t, dt,
                                         as_device(q_pts, self.mesh.device))
