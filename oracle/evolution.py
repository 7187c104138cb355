"""Time integrators and the CMM map update (oracle restatement of
cmm_s2/core/evolution_functions.py)."""
import numpy as np
from .geometry import unit_rows
from .spline import MapOracle


def _proj(x):
    """div_norm (cmm_s2/core/evolution_functions.py:82-85); x (3,N)."""
    return (1 / np.sqrt(x[0] ** 2 + x[1] ** 2 + x[2] ** 2))[None] * x


def euler_back(t, dt, x, V):
    """Euler_step_proj (:19-23)."""
    return _proj(x - dt * V(t, dt, x))


def improved_euler_back(t, dt, x, V):
    """improved_Euler_proj (:25-33)."""
    v1 = V(t, dt, x)
    s1 = _proj(x - dt * v1)
    v2 = V(t + dt, dt, s1)
    return _proj(x - (dt / 2) * (v1 + v2))


def rk4_back(t, dt, x, V):
    """RK4_proj (:50-67): backward RK4, each stage projected onto the sphere."""
    v1 = V(t + dt, dt, x)
    s1 = _proj(x - dt * v1 / 2)
    v2 = V(t + dt / 2, dt, s1)
    s2 = _proj(x - (dt / 2) * v2)
    v3 = V(t + 0.5 * dt, dt, s2)
    s3 = _proj(x - dt * v3)
    v4 = V(t, dt, s3)
    return _proj(x - (dt / 6) * (v1 + 2 * v2 + 2 * v3 + v4))


def rk2_back(t, dt, x, V):
    """RK2_proj (:68-78)."""
    v1 = V(t + dt, dt, x)
    s1 = _proj(x - (dt / 2) * v1)
    v2 = V(t + dt / 2, dt, s1)
    return _proj(x - dt * v2)


def jets_from_stencil(s_evals, tan, eps=1e-5):
    """spline_proj_sphere (:90-113): new jets (3,4,Nv) from the 4 stencil
    images s_evals (3,4,Nv) and the vertex tangent frames tan (2,Nv,3)."""
    nv = s_evals.shape[2]
    jets = np.empty((3, 4, nv))
    m = (s_evals[:, 0] + s_evals[:, 1] + s_evals[:, 2] + s_evals[:, 3]) / 4
    jets[:, 0] = unit_rows(m.T).T
    d1 = (s_evals[:, 1] - s_evals[:, 0] + s_evals[:, 3] - s_evals[:, 2]) / (4 * eps)
    d2 = (s_evals[:, 2] - s_evals[:, 0] + s_evals[:, 3] - s_evals[:, 1]) / (4 * eps)
    for k in range(3):
        jets[:, 1 + k] = (d1[k][:, None] * tan[0] + d2[k][:, None] * tan[1]).T
    return jets


def advect_project(prev_map, integrator, t, dt, V, verts, s_pts, tan, identity):
    """advect + spline_proj_sphere (:117-142): the jets of the next map.

    prev_map: a MapOracle (ignored when identity is True)."""
    yn = integrator(t, dt, verts.T, V)
    s = s_pts.shape
    sn = integrator(t, dt, s_pts.reshape(3, s[1] * s[2]), V).reshape(s)
    if not identity:
        sn = prev_map.stencil_eval(yn, sn)
    return jets_from_stencil(sn, tan)


def identity_jets(verts):
    """Identity map jets (cmm_s2/core/spherical_simulations.py:165-169)."""
    x = verts.T
    jets = np.zeros((3, 4, len(verts)))
    jets[:, 0] = x
    for k in range(3):
        e = np.zeros((3, 1)); e[k] = 1.0
        # utils.tan_proj(x, e_k) (cmm_s2/core/utils.py:29-34, 87-94)
        g = np.array([(1 - x[0] ** 2) * e[0] + (-x[0] * x[1]) * e[1] + (-x[0] * x[2]) * e[2],
                      (-x[0] * x[1]) * e[0] + (1 - x[1] ** 2) * e[1] + (-x[1] * x[2]) * e[2],
                      (-x[0] * x[2]) * e[0] + (-x[1] * x[2]) * e[1] + (1 - x[2] ** 2) * e[2]])
        jets[k, 1:] = g
    return jets
