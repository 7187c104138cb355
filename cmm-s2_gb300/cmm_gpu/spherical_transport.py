"""Linear advection of a tracer on the sphere by the CMM: the time loop of
cmm_s2/tests/test_spherical_transport.py (advect_project_sphere under an
analytic flow, optional remapping every ``n_maps`` steps, evaluation of the
tracer through the composed maps), on libcmmgpu.so.

Each step is one cmm_flow_advect_project call (foot points of the vertices
and stencil points under the closed-form flow, then the new jets from the
stencil images through the previous map) and one assembly of the new
submap's coefficients.  Remapped submaps keep their own coefficient
records; the reference's test loop re-uses the first map object after a
remap, so every remap it stores shares one coefficient array
(evolution_functions.py:113 aliasing), which this driver does not copy.
"""
import numpy as np
import torch

from . import native
from .dynamical_fields import Flow
from .evolution_functions import RK4_proj, _SCHEMES
from .meshgen import icosahedral_mesh, identity_jets
from .mesh_functions import as_device, spherical_triangulation
from .spherical_spline import sphere_diffeomorphism


class TransportSolver:
    """CMM linear transport: `U` an analytic flow of cmm_gpu.dynamical_fields,
    final time T over Nt steps (tspan = linspace(0, T, Nt, endpoint=False),
    dt = tspan[1] - tspan[0], as the reference's loop)."""

    def __init__(self, mesh, U, T=1.0, Nt=None, integrator=RK4_proj, remapping=False, n_maps=10, device=None):
        if not isinstance(U, Flow):
            raise TypeError("U must be an analytic flow of cmm_gpu.dynamical_fields")
        if isinstance(mesh, int):
            v, t = icosahedral_mesh(mesh)
            mesh = spherical_triangulation(v, t, device=device)
        self.mesh, self.U, self.T = mesh, U, float(T)
        self.Nt = 2 ** mesh.level + 10 if Nt is None else int(Nt)
        self.tspan = np.linspace(0, self.T, self.Nt, endpoint=False)
        self.dt = float(self.tspan[1] - self.tspan[0])
        self.scheme = _SCHEMES[integrator]
        self.remapping, self.n_maps = remapping, int(n_maps)
        self.jet0 = torch.from_numpy(identity_jets(mesh.vertices)).to(mesh.device)
        self.remaps = []
        self.mapping = sphere_diffeomorphism(mesh, self.jet0.clone())
        self.identity = True
        self.count = 0
        self._work = torch.empty(native.lib.cmm_advect_workspace(mesh.native.h), dtype=torch.float64,
                                 device=mesh.device)

    def step(self):
        """One step of the loop (test_spherical_transport.py:98-107)."""
        t = float(self.tspan[self.count])
        nat = self.mesh.native
        jets = torch.empty((3, 4, nat.nv), dtype=torch.float64, device=self.mesh.device)
        nat.flow_advect_project(self.U.kind, self.scheme, t, self.dt, self.mesh.s_pts_d, self.mesh.tan_d,
                                None if self.identity else self.mapping.coeffs, T=self.U.T, alpha=self.U.alpha,
                                jets=jets, work=self._work)
        self.mapping = sphere_diffeomorphism(self.mesh, jets, self.mapping.coeffs)
        self.identity = False
        self.count += 1
        if self.remapping and self.count % self.n_maps == 0:
            self.remaps.append(self.mapping)
            self.mapping = sphere_diffeomorphism(self.mesh, self.jet0.clone())
            self.identity = True
        return self

    def run(self, nsteps=None):
        n = self.Nt - self.count if nsteps is None else nsteps
        for _ in range(n):
            self.step()
        return self

    def maps(self):
        """The submaps, first remap first (the reference's list after the
        loop: remaps plus the current map unless it is the identity)."""
        return self.remaps + ([] if self.identity else [self.mapping])

    def __call__(self, q):
        """Backward characteristic map X(q) (N,3) -> (N,3): the submaps
        composed last-first (compose_maps, evolution_functions.py:147-153)."""
        maps = self.maps()
        q = as_device(q, self.mesh.device)
        if not maps:
            return q.clone()
        return self.mesh.native.compose([m.coeffs for m in maps], q)[0]

    def tracer(self, q, kind=native.TRACER_SMOOTH_TEST, t=0.0):
        """Transported tracer h0(X(q)) at q (N,3)."""
        return self.mesh.native.tracer(kind, self(q), t=t)

    def error(self, q, kind=native.TRACER_SMOOTH_TEST, exact=None):
        """max |h0(X(q)) - exact| with exact = h0(q) by default (the flows of
        the reference's test return every particle at t = T)."""
        q = as_device(q, self.mesh.device)
        ref = self.mesh.native.tracer(kind, q) if exact is None else as_device(exact, self.mesh.device)
        return float((self.tracer(q, kind) - ref).abs().max())
