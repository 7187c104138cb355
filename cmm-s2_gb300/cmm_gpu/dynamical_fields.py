"""Linear-transport test flows and tracer fields with the names and call
signatures of cmm_s2/core/dynamical_fields.py, evaluated by libcmmgpu.so.

The flows are objects callable as ``U(t, dt, X)`` with X (3,N), like the
reference's functions; handed to ``evolution_functions.advect_project_sphere``
or the integrators of this package they are evaluated in closed form inside
the CUDA integrators (no velocity mesh).  The module constants ``T`` (period)
and ``alpha`` (tilt of the solid-body rotation) are read at call time, as
the reference reads its module globals.
"""
import numpy as np
import torch

from . import native
from .mesh_functions import as_device

pi = np.pi
T = 1
alpha = 0

_STATUS = {}


def _status_mesh(device):
    """A level-0 icosahedral mesh per device whose status word records
    non-finite results of the point evaluations."""
    if device not in _STATUS:
        from .meshgen import icosahedral_mesh
        v, t = icosahedral_mesh(0)
        _STATUS[device] = native.Mesh(v, t, 0, device=device.index)
    return _STATUS[device]


def _device_of(X):
    if isinstance(X, torch.Tensor) and X.is_cuda:
        return X.device
    return torch.device("cuda", torch.cuda.current_device())


class Flow:
    """One analytic velocity field (dynamical_fields.py:18-107)."""

    def __init__(self, kind, name):
        self.kind, self.__name__ = kind, name

    @property
    def T(self):
        return float(T)

    @property
    def alpha(self):
        return float(alpha)

    def __call__(self, t, dt, X):
        dev = _device_of(X)
        x = as_device(X, dev)
        return _status_mesh(dev).flow_velocity(self.kind, float(t), x, T=self.T, alpha=self.alpha)

    def __repr__(self):
        return f"<flow {self.__name__}>"


u_sbr = Flow(native.FLOW_SOLID_BODY, "u_sbr")                        # :18-22
u_deform = Flow(native.FLOW_DEFORM, "u_deform")                      # :24-30
u_deform_rot = Flow(native.FLOW_DEFORM_ROT, "u_deform_rot")          # :32-42
u_static_vortex = Flow(native.FLOW_STATIC_VORTEX, "u_static_vortex")  # :57-65
u_rotating_vortex = Flow(native.FLOW_ROTATING_VORTEX, "u_rotating_vortex")  # :67-76
equator_vortex = Flow(native.FLOW_EQUATOR_VORTEX, "equator_vortex")  # :78-83
u_div = Flow(native.FLOW_DIVERGENT, "u_div")                         # :97-107


def _tracer_xyz(kind, xyz, t=0.0):
    """Tracer at points xyz (3,N) (any trailing shape)."""
    dev = _device_of(xyz)
    x = as_device(xyz, dev)
    shape = x.shape[1:]
    pts = x.reshape(3, -1).T.contiguous()
    return _status_mesh(dev).tracer(kind, pts, t=float(t)).reshape(shape)


def _tracer_angles(kind, phi, theta):
    dev = _device_of(phi)
    phi, theta = as_device(phi, dev), as_device(theta, dev)
    xyz = torch.stack([torch.sin(theta) * torch.cos(phi), torch.sin(theta) * torch.sin(phi), torch.cos(theta)])
    return _tracer_xyz(kind, xyz)


def cosine_bell(phi, theta):
    """Two cosine bells (:122-137)."""
    return _tracer_angles(native.TRACER_COSINE_BELL, phi, theta)


def IC_SC(phi, theta):
    """Two slotted cylinders (:139-157)."""
    return _tracer_angles(native.TRACER_SLOTTED_CYLINDERS, phi, theta)


def static_vort_IC(t, xyz):
    """Exact tracer of the static vortex at time t (:85-88)."""
    return _tracer_xyz(native.TRACER_STATIC_VORTEX, xyz, t)


def rotating_vort_IC(t, xyz):
    """Tracer of the rotating vortex (:90-95)."""
    return _tracer_xyz(native.TRACER_ROTATING_VORTEX, xyz, t)


def smooth_test(xyz):
    """The smooth test function of tests/test_spherical_transport.py:36-38 at
    points xyz (N,3)."""
    dev = _device_of(xyz)
    return _status_mesh(dev).tracer(native.TRACER_SMOOTH_TEST, as_device(xyz, dev))


def random_initial_condition(xyz):
    """The random smooth field of :158-172 at points xyz (3,N): the series
    sum_{1<=l<=32, -l<=m<l} c_lm Re Y_l^m with c numpy's seed-42 uniform(-1, 1)
    draws, the coefficients regenerated inside the library (MT19937)."""
    return _tracer_xyz(native.TRACER_RANDOM_SH, xyz)
