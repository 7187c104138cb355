"""Reference FP64 gradient of the vorticity at the back-traced points (test
infrastructure).

TEST INFRASTRUCTURE ONLY, like the rest of ``oracle``: a pure-torch FP64
restatement of ``oracle.fields.sh_series`` (the real orthonormal series of
the initial vorticity, cmm_s2/core/dynamical_fields.py:181-214 with the
coefficient layout of cmm_s2/core/spherical_harmonic_tools.py:30-47) plus
the planetary term of the sampled vorticity, omega = omega0(X) +
2 Omega cos theta(X) - 2 Omega cos theta (cmm_s2/core/spherical_simulations.py:
269-272), so that torch autograd on the CPU gives an independent gradient
with respect to the series coefficients and to the points X.  The points
are projected onto the sphere inside the restatement, which makes it
invariant to their scale, so its point gradient is tangent.
"""
import math

import torch


def sh_series_at(coeffs, X):
    """omega0 at points X (N,3): coeffs (lmax+1, 2 lmax+1), column l + m."""
    lmax = coeffs.shape[0] - 1
    P = X / torch.sqrt((X * X).sum(1, keepdim=True))
    x = P[:, 2]
    s = torch.sqrt(P[:, 0] ** 2 + P[:, 1] ** 2)
    phi = torch.atan2(P[:, 1], P[:, 0])
    out = torch.zeros_like(x)
    pmm = torch.full_like(x, math.sqrt(1 / (4 * math.pi)))
    for m in range(lmax + 1):
        if m > 0:
            pmm = -pmm * math.sqrt((2 * m + 1) / (2 * m)) * s
        p_prev, p = None, pmm
        for l in range(m, lmax + 1):
            if l == m + 1:
                p_prev, p = p, math.sqrt(2 * m + 3) * x * pmm
            elif l > m + 1:
                a = math.sqrt((4 * l * l - 1) / (l * l - m * m))
                b = math.sqrt(((l - 1) ** 2 - m * m) / (4 * (l - 1) ** 2 - 1))
                p_prev, p = p, a * (x * p - b * p_prev)
            if m == 0:
                out = out + coeffs[l, l] * p
            else:
                out = out + math.sqrt(2) * p * (coeffs[l, l + m] * torch.cos(m * phi)
                                                + coeffs[l, l - m] * torch.sin(m * phi))
    return out


def sampled_vorticity(coeffs, X, rot_rate, cos_theta_grid):
    """omega0(X) + 2 Omega cos theta(X) - 2 Omega cos theta_grid, flat (N,)."""
    z = X[:, 2] / torch.sqrt((X * X).sum(1))
    return sh_series_at(coeffs, X) + 2 * rot_rate * z - 2 * rot_rate * cos_theta_grid
