"""Reference FP64 gradient of the submap composition (test infrastructure).

TEST INFRASTRUCTURE ONLY, like the rest of ``oracle``: a pure-torch FP64
restatement of ``composite_sphere_diffeomorphism.__call__``
(cmm_s2/core/spherical_spline.py:365-398, applied submap S-1 first, submap 0
last) built from the numpy oracle's pieces, so that torch autograd on the
CPU gives an independent gradient of the composed points with respect to
the ordinates of every submap and to the query points.

Per submap the evaluation is the one of ``oracle.spline.eval_patch`` with
``closed=True``: big-triangle barycentrics b = R p (``inverse_rows``), the
Powell-Sabin sub-triangle (argmin b, argmax b) of
cmm_s2/core/spherical_spline.py:668-697, its barycentrics in closed form
(``split_bary_closed``), the six-ordinate quadratic Bernstein-Bezier sum
(:178-205) and the projection onto the sphere.  The piecewise choices (the
containing triangle, found by the oracle's locator, and the sub-triangle)
are made on the forward points and held fixed; everything else is a torch
operation on the differentiated tensors.
"""
import numpy as np
import torch

from .geometry import query
from .spline import SPLIT_CORNERS, SPLIT_ORDINATES, inverse_rows


def submap_eval(coeffs, p, verts, tris, locator):
    """One submap: coeffs (3,19,Nt) and points p (N,3), both FP64 torch
    tensors (either may require grad) -> normalised images (N,3)."""
    pn = p.detach().cpu().numpy()
    _, tri, vs = query(verts, tris, locator, pn)
    if (tri < 0).any():
        raise ValueError("a point lies outside the mesh (non-finite?)")
    R = inverse_rows(vs)
    bb_np = np.einsum("nij,nj->ni", R, pn)
    lo, hi = np.argmin(bb_np, axis=1), np.argmax(bb_np, axis=1)
    n = np.arange(len(pn))
    mid = 3 - lo - hi
    N4 = torch.from_numpy(np.linalg.norm(vs.sum(1), axis=1))
    Ne = torch.from_numpy(np.linalg.norm(vs[n, hi] + vs[n, mid], axis=1))
    bb = torch.einsum("nij,nj->ni", torch.from_numpy(R), p)
    nt = torch.from_numpy(n)
    lo_t, hi_t, mid_t = torch.from_numpy(lo), torch.from_numpy(hi), torch.from_numpy(mid)
    gV = bb[nt, hi_t] - bb[nt, mid_t]
    gE = Ne * (bb[nt, mid_t] - bb[nt, lo_t])
    gC = N4 * bb[nt, lo_t]
    corn = torch.from_numpy(SPLIT_CORNERS[lo, hi])              # (N,3) pool ids
    b = [torch.where(corn[:, k] == hi_t, gV, torch.where(corn[:, k] == 3, gC, gE)) for k in range(3)]
    ords = torch.from_numpy(SPLIT_ORDINATES[lo, hi])           # (N,6)
    cf = coeffs[:, ords, torch.from_numpy(tri)[:, None]]       # (3,N,6)
    val = (b[0] ** 2 * cf[..., 0] + b[1] ** 2 * cf[..., 1] + b[2] ** 2 * cf[..., 2]
           + 2 * b[1] * b[0] * cf[..., 3] + 2 * b[2] * b[1] * cf[..., 4] + 2 * b[2] * b[0] * cf[..., 5])
    return (val / torch.sqrt((val * val).sum(0))).T


def composite_eval(coeff_stack, q, verts, tris, locator):
    """Composition X = S_0 o ... o S_{S-1}(q): coeff_stack a list of (3,19,Nt)
    FP64 tensors (submap 0 first), q (N,3) -> (N,3)."""
    p = q
    for c in reversed(coeff_stack):
        p = submap_eval(c, p, verts, tris, locator)
    return p
