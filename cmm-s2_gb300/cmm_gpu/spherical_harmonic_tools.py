"""Spherical-harmonic tools with the interface of
cmm_s2/core/spherical_harmonic_tools.py, backed by libcmmgpu.so.

Coefficients are exchanged in the reference's (L, 2L+1) "shifted" layout
(row l, column m + l; coeff_array, :30-42) as complex128 CUDA tensors.
The library works in an m-major half layout (m >= 0) and applies the
exact ladder operators; the L_plus/L_minus/L_z arguments are accepted for
signature compatibility and must be the reference's standard operators
(spherical_simulations.py:201-205)."""
import numpy as np
import torch

from . import native
from .mesh_functions import as_device

_PLANS = {}


def plan(L, device=None):
    dev = device or torch.device("cuda", torch.cuda.current_device())
    key = (L, dev)
    if key not in _PLANS:
        _PLANS[key] = native.Sht(L, device=dev.index)
    return _PLANS[key]


def _index(L, device):
    l = torch.arange(L, device=device)[:, None]
    m = torch.arange(2 * L + 1, device=device)[None, :] - l      # m of each shifted column
    valid = m.abs() <= l
    return l, m, valid


def half_to_shifted(alm, L):
    """m-major half layout (L,L) [m,l] -> shifted (L, 2L+1) [l, l+m]."""
    l, m, valid = _index(L, alm.device)
    ma = m.abs().clamp(max=L - 1)
    a = alm[ma, l.expand_as(ma)]
    neg = (m < 0)
    sign = torch.where(ma % 2 == 1, -1.0, 1.0).to(torch.float64)
    a = torch.where(neg, sign * a.conj(), a)
    return torch.where(valid, a, torch.zeros((), dtype=a.dtype, device=a.device))


def shifted_to_half(c, L):
    """shifted (L, 2L+1) -> m-major half (L,L) [m,l] (m >= 0 columns)."""
    m = torch.arange(L, device=c.device)[:, None]
    l = torch.arange(L, device=c.device)[None, :]
    col = (l + m).clamp(max=2 * L)
    out = c[l.expand(L, L), col]
    return torch.where(m <= l, out, torch.zeros((), dtype=out.dtype, device=out.device)).contiguous()


def coeff_array(alms, L):
    """pyssht 1-D vector (L*L,) -> shifted layout (:30-42)."""
    alms = torch.as_tensor(alms)
    out = torch.zeros((L, 2 * L + 1), dtype=torch.complex128, device=alms.device)
    for l in range(L):
        out[l, :2 * l + 1] = alms[l * l: l * l + 2 * l + 1]
    return out


def lm_array(coeffs, L):
    """shifted layout -> pyssht 1-D vector (:44-47)."""
    return torch.cat([coeffs[l, :2 * l + 1] for l in range(L)])


def inv_Laplacian(samples, L, L_inv):
    """Forward MWSS transform times D_inv, shifted layout (:14-19)."""
    s = as_device(samples)
    alm = plan(L, s.device).forward(s)
    d = torch.as_tensor(np.asarray(L_inv), dtype=torch.float64, device=s.device)
    return half_to_shifted(alm, L) * d[:, None]


def project_stream(alms, L, L_plus, L_minus, L_z, U, n, temp=None):
    """Velocity jets of the stream function into time level n of U (:66-105)."""
    if U.stepping:
        U.coeffs[0], U.coeffs[1], U.coeffs[2] = U.coeffs[1], U.coeffs[2], U.coeffs[0]
        U.vals[0:2] = U.vals[1:3].clone()
    psi = shifted_to_half(torch.as_tensor(alms, device=U.mesh.device).to(torch.complex128), L)
    jets = torch.empty((3, 4, U.mesh.native.nv), dtype=torch.float64, device=U.mesh.device)
    native.check(native.lib.cmm_sht_velocity(plan(L, U.mesh.device).h, U.mesh.native.h, None,
                                             native._ptr(psi), native._ptr(jets),
                                             native._stream(U.mesh.device)), "cmm_sht_velocity")
    U.vals[n] = jets
    U.init_coeffs(n)
