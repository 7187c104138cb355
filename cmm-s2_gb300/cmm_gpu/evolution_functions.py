"""Backward integrators and the CMM map update with the interface of
cmm_s2/core/evolution_functions.py, backed by libcmmgpu.so.  ``V`` must be
a spline_interp_velocity of this package."""
import torch

from . import native
from .mesh_functions import as_device
from .spherical_spline import sphere_diffeomorphism


def _integrate(scheme, t, dt, xn, V):
    return V.mesh.native.integrate(V.coeffs[:V.nVs], float(V.ts[0]), scheme, t, dt,
                                   as_device(xn, V.mesh.device))


def Euler_step_proj(t, dt, xn, V):
    """:19-23"""
    return _integrate(native.EULER, t, dt, xn, V)


def improved_Euler_proj(t, dt, xn, V):
    """:25-33"""
    return _integrate(native.IMPROVED_EULER, t, dt, xn, V)


def RK4_proj(t, dt, xn, V):
    """:50-67"""
    return _integrate(native.RK4, t, dt, xn, V)


_SCHEMES = {Euler_step_proj: native.EULER, improved_Euler_proj: native.IMPROVED_EULER,
            RK4_proj: native.RK4}


def advect_project_sphere(interp, integrator, t, dt, V, identity=False):
    """advect + spline_proj_sphere (:117-142) as one library call: returns
    the next map, whose coefficients overwrite ``interp.coeffs`` (the
    reference shares that array the same way, :113)."""
    mesh = interp.mesh
    jets = torch.empty((3, 4, mesh.native.nv), dtype=torch.float64, device=mesh.device)
    mesh.native.advect_project(V.mesh.native, V.coeffs[:V.nVs], float(V.ts[0]), _SCHEMES[integrator],
                               t, dt, mesh.s_pts_d, mesh.tan_d, None if identity else interp.coeffs,
                               jets=jets)
    return sphere_diffeomorphism(mesh, jets, interp.coeffs)
