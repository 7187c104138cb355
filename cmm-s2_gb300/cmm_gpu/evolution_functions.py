"""Backward integrators and the CMM map update with the interface of
cmm_s2/core/evolution_functions.py, backed by libcmmgpu.so.  ``V`` is a
spline_interp_velocity of this package or one of the analytic flows of
cmm_gpu.dynamical_fields (u_sbr, u_deform_rot, ...)."""
import torch

from . import native
from .dynamical_fields import Flow, _status_mesh
from .mesh_functions import as_device
from .spherical_spline import sphere_diffeomorphism


def _integrate(scheme, t, dt, xn, V):
    if isinstance(V, Flow):
        dev = xn.device if isinstance(xn, torch.Tensor) and xn.is_cuda else \
            torch.device("cuda", torch.cuda.current_device())
        return _status_mesh(dev).flow_integrate(V.kind, scheme, float(t), float(dt), as_device(xn, dev),
                                                T=V.T, alpha=V.alpha)
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


def RK2_proj(t, dt, xn, V):
    """:68-78"""
    return _integrate(native.RK2, t, dt, xn, V)


_SCHEMES = {Euler_step_proj: native.EULER, improved_Euler_proj: native.IMPROVED_EULER,
            RK4_proj: native.RK4, RK2_proj: native.RK2}


def advect_project_sphere(interp, integrator, t, dt, V, identity=False):
    """advect + spline_proj_sphere (:117-142) as one library call: returns
    the next map, whose coefficients overwrite ``interp.coeffs`` (the
    reference shares that array the same way, :113)."""
    mesh = interp.mesh
    jets = torch.empty((3, 4, mesh.native.nv), dtype=torch.float64, device=mesh.device)
    if isinstance(V, Flow):
        mesh.native.flow_advect_project(V.kind, _SCHEMES[integrator], float(t), float(dt), mesh.s_pts_d,
                                        mesh.tan_d, None if identity else interp.coeffs, T=V.T,
                                        alpha=V.alpha, jets=jets)
        return sphere_diffeomorphism(mesh, jets, interp.coeffs)
    mesh.native.advect_project(V.mesh.native, V.coeffs[:V.nVs], float(V.ts[0]), _SCHEMES[integrator],
                               t, dt, mesh.s_pts_d, mesh.tan_d, None if identity else interp.coeffs,
                               jets=jets)
    return sphere_diffeomorphism(mesh, jets, interp.coeffs)


def compose_maps(remaps, evals, current=[]):
    """compose_maps (:147-153): the maps of ``remaps + current`` applied
    last-first to evals (N,3) -> (N,3), as one composition launch."""
    maps = list(remaps) + list(current)
    if not maps:
        return as_device(evals).clone()
    mesh = maps[0].mesh
    out, _, _, _ = mesh.native.compose([m.coeffs for m in maps], as_device(evals, mesh.device))
    return out
