"""Powell-Sabin spline maps, composition, velocity interpolant, Jacobians
(oracle restatement of cmm_s2/core/spherical_spline.py)."""
import numpy as np
from .geometry import bary, query, ps_split, unit_rows

# Ordinate ids of the quadratic Bezier patch on each Powell-Sabin
# sub-triangle, indexed [argmin bcc][argmax bcc]
# (the table of cmm_s2/core/spherical_spline.py:660-662).
SPLIT_ORDINATES = np.array([[[0, 0, 0, 0, 0, 0], [18, 1, 13, 7, 6, 16], [13, 2, 18, 11, 10, 16]],
                            [[18, 14, 0, 17, 5, 4], [0, 0, 0, 0, 0, 0], [14, 18, 2, 17, 10, 9]],
                            [[0, 12, 18, 3, 15, 4], [1, 18, 12, 7, 15, 8], [0, 0, 0, 0, 0, 0]]])
# Sub-triangle corners drawn from (v1,v2,v3,v4,e1,e2,e3), same indexing
# (cmm_s2/core/spherical_spline.py:664-666).
SPLIT_CORNERS = np.array([[[0, 0, 0], [3, 1, 5], [5, 2, 3]],
                          [[3, 6, 0], [0, 0, 0], [6, 3, 2]],
                          [[0, 4, 3], [1, 3, 4], [0, 0, 0]]])


def assemble(verts, tris, vals, geom=None):
    """19 quadratic Bezier ordinates per triangle from per-vertex jets
    (sphere_diffeomorphism.assemble_coefficients,
    cmm_s2/core/spherical_spline.py:300-337).

    vals: (C,4,Nv) with vals[c,0] = f_c and vals[j,1+k] = d_j f_k (the
    reference's jet layout).  Returns coeffs (C,19,Nt)."""
    H, G, E = geom if geom is not None else ps_split(verts, tris)
    C = vals.shape[0]
    tv = vals[:, :, tris]              # (C,4,Nt,3)
    out = np.zeros((C, 19, len(tris)))
    out[:, 0], out[:, 1], out[:, 2] = tv[:, 0, :, 0], tv[:, 0, :, 1], tv[:, 0, :, 2]

    def grad_ord(h, g, gi, corner):
        # sum_j h_j * vals[j, 1+k] -> component k
        dot = h[:, 0] * tv[0, 1:, :, corner] + h[:, 1] * tv[1, 1:, :, corner] + h[:, 2] * tv[2, 1:, :, corner]
        return (1 / g[:, gi])[None] * (dot / 2 - g[:, 0][None] * tv[:, 0, :, corner])

    out[:, 3] = grad_ord(H[0], G[0], 1, 0)
    out[:, 4] = grad_ord(H[6], G[6], 1, 0)
    out[:, 5] = grad_ord(H[4], G[4], 2, 0)
    out[:, 6] = grad_ord(H[2], G[2], 1, 1)
    out[:, 7] = grad_ord(H[7], G[7], 1, 1)
    out[:, 8] = grad_ord(H[1], G[1], 2, 1)
    out[:, 9] = grad_ord(H[5], G[5], 1, 2)
    out[:, 10] = grad_ord(H[8], G[8], 1, 2)
    out[:, 11] = grad_ord(H[3], G[3], 2, 2)
    e1, e2, e3, mid = E[0], E[1], E[2], G[9]
    out[:, 12] = e1[:, 0] * out[:, 3] + e1[:, 1] * out[:, 8]
    out[:, 13] = e2[:, 1] * out[:, 6] + e2[:, 2] * out[:, 11]
    out[:, 14] = e3[:, 2] * out[:, 9] + e3[:, 0] * out[:, 5]
    out[:, 15] = e1[:, 0] * out[:, 4] + e1[:, 1] * out[:, 7]
    out[:, 16] = e2[:, 1] * out[:, 7] + e2[:, 2] * out[:, 10]
    out[:, 17] = e3[:, 0] * out[:, 4] + e3[:, 2] * out[:, 10]
    out[:, 18] = mid[:, 0] * out[:, 4] + mid[:, 1] * out[:, 7] + mid[:, 2] * out[:, 10]
    return out


def assemble_scalar(verts, tris, vals, geom=None):
    """spherical_spline.assemble_coefficients (cmm_s2/core/spherical_spline.py:
    115-152): vals (4,Nv) = value, gradient -> coeffs (19,Nt)."""
    H, G, E = geom if geom is not None else ps_split(verts, tris)
    tv = vals[:, tris]                 # (4,Nt,3)
    out = np.zeros((19, len(tris)))
    out[0], out[1], out[2] = tv[0, :, 0], tv[0, :, 1], tv[0, :, 2]

    def grad_ord(h, g, gi, corner):
        dot = h[:, 0] * tv[1, :, corner] + h[:, 1] * tv[2, :, corner] + h[:, 2] * tv[3, :, corner]
        return (1 / g[:, gi]) * (dot / 2 - g[:, 0] * tv[0, :, corner])

    spec = [(3, 0, 1, 0), (4, 6, 1, 0), (5, 4, 2, 0), (6, 2, 1, 1), (7, 7, 1, 1), (8, 1, 2, 1),
            (9, 5, 1, 2), (10, 8, 1, 2), (11, 3, 2, 2)]
    for o, k, gi, corner in spec:
        out[o] = grad_ord(H[k], G[k], gi, corner)
    e1, e2, e3, mid = E[0], E[1], E[2], G[9]
    out[12] = e1[:, 0] * out[3] + e1[:, 1] * out[8]
    out[13] = e2[:, 1] * out[6] + e2[:, 2] * out[11]
    out[14] = e3[:, 2] * out[9] + e3[:, 0] * out[5]
    out[15] = e1[:, 0] * out[4] + e1[:, 1] * out[7]
    out[16] = e2[:, 1] * out[7] + e2[:, 2] * out[10]
    out[17] = e3[:, 0] * out[4] + e3[:, 2] * out[10]
    out[18] = mid[:, 0] * out[4] + mid[:, 1] * out[7] + mid[:, 2] * out[10]
    return out


def split_corners(vs, bcc, tie_fix=False):
    """Sub-triangle corners (new_vpoints, cmm_s2/core/spherical_spline.py:668-697).

    With tie_fix, a query at the split centre (all bcc equal, where the
    reference's tables select no sub-triangle and it returns 0/0) uses the
    sub-triangle (argmin, argmax) = (1, 0) instead."""
    v1, v2, v3 = vs[:, 0], vs[:, 1], vs[:, 2]
    e1, e2, e3 = unit_rows(v1 / 2 + v2 / 2), unit_rows(v2 / 2 + v3 / 2), unit_rows(v3 / 2 + v1 / 2)
    v4 = unit_rows((v1 + v2 + v3) / 3)
    pool = np.stack([v1, v2, v3, v4, e1, e2, e3])          # (7,N,3)
    lo, hi = np.argmin(bcc, axis=1), np.argmax(bcc, axis=1)
    if tie_fix:
        tie = lo == hi
        lo, hi = np.where(tie, 1, lo), np.where(tie, 0, hi)
    js = SPLIT_CORNERS[lo, hi]                               # (N,3)
    n = np.arange(len(bcc))
    return np.stack([pool[js[:, 0], n], pool[js[:, 1], n], pool[js[:, 2], n]], 1), lo, hi


def _sbb(cf, b):
    """Quadratic Bernstein-Bezier sum over the 6 ordinates (cf (...,6,N))."""
    return ((b[:, 0] ** 2) * cf[..., 0, :] + (b[:, 1] ** 2) * cf[..., 1, :] + (b[:, 2] ** 2) * cf[..., 2, :]
            + 2 * (b[:, 1] * b[:, 0]) * cf[..., 3, :] + 2 * (b[:, 2] * b[:, 1]) * cf[..., 4, :]
            + 2 * (b[:, 2] * b[:, 0]) * cf[..., 5, :])


def inverse_rows(vs):
    """Rows of the inverse vertex matrix of each triangle, (N,3,3):
    bcc = R q with R = [v2 x v3, v3 x v1, v1 x v2] / det(v1,v2,v3)."""
    v1, v2, v3 = vs[:, 0], vs[:, 1], vs[:, 2]
    from .geometry import det_cols
    d = det_cols(v1, v2, v3)
    return np.stack([np.cross(v2, v3), np.cross(v3, v1), np.cross(v1, v2)], 1) / d[:, None, None]


def split_bary_closed(vs, R, pts, lo, hi):
    """Sub-triangle barycentrics of pts in closed form, (N,3) in the corner
    order of SPLIT_CORNERS[lo, hi].

    The reference's new_vpoints + bary_coords (cmm_s2/core/spherical_spline.py:
    668-689, cmm_s2/core/utils.py:58-67) compute them from four determinants
    per point.  The sub-triangle's corners are v_hi, e = (v_hi+v_mid)/|.| and
    c = (v1+v2+v3)/|.|, so the same linear map is
        g_V = b_hi - b_mid,  g_E = |v_hi+v_mid| (b_mid - b_lo),  g_C = |v1+v2+v3| b_lo
    with b = R pts the big-triangle barycentrics.  This evaluation shares its
    rounding between nearby points (the finite-difference jets of
    cmm_s2/core/evolution_functions.py:102-103 then do not amplify it)."""
    n = np.arange(len(pts))
    b = np.einsum("nij,nj->ni", R, pts)
    mid = 3 - lo - hi
    v = [vs[:, 0], vs[:, 1], vs[:, 2]]
    N4 = np.linalg.norm(vs[:, 0] + vs[:, 1] + vs[:, 2], axis=1)
    Ne = np.linalg.norm(np.stack(v)[hi, n] + np.stack(v)[mid, n], axis=1)
    gV, gE, gC = b[n, hi] - b[n, mid], Ne * (b[n, mid] - b[n, lo]), N4 * b[n, lo]
    corn = SPLIT_CORNERS[lo, hi]
    out = np.empty((len(pts), 3))
    for p in range(3):
        c = corn[:, p]
        out[:, p] = np.where(c == hi, gV, np.where(c == 3, gC, gE))
    return out


def eval_patch(coeffs, tri, bcc_big, vs, pts, tie_fix=False, closed=False):
    """Evaluate un-normalised patches at ``pts`` located in ``tri`` with
    big-triangle bcc ``bcc_big``; coeffs (...,19,Nt).  Returns (...,N).
    closed=True uses split_bary_closed for the sub-triangle barycentrics."""
    if closed:
        R = inverse_rows(vs)
        bcc_big = np.einsum("nij,nj->ni", R, pts)
    vn, lo, hi = split_corners(vs, bcc_big, tie_fix)
    ords = SPLIT_ORDINATES[lo, hi]
    if closed:
        b = split_bary_closed(vs, R, pts, lo, hi)
    else:
        b = bary(vn[:, 0], vn[:, 1], vn[:, 2], pts)
    cf = np.stack([coeffs[..., ords[:, k], tri] for k in range(6)], axis=-2)
    return _sbb(cf, b)


class MapOracle:
    """sphere_diffeomorphism (cmm_s2/core/spherical_spline.py:155-337)."""

    def __init__(self, verts, tris, locator, vals, geom=None, tie_fix=False, closed=False):
        self.verts, self.tris, self.loc = verts, tris, locator
        self.tie_fix, self.closed = tie_fix, closed
        self.vals = vals
        self.coeffs = assemble(verts, tris, vals, geom)

    def __call__(self, q):
        """__call__ (:178-205): normalised image, (3,N)."""
        bcc, tri, vs = query(self.verts, self.tris, self.loc, q)
        out = eval_patch(self.coeffs, tri, bcc, vs, q, self.tie_fix, self.closed)
        nrm = np.sqrt(out[0] ** 2 + out[1] ** 2 + out[2] ** 2)
        return (1 / nrm)[None] * out

    def stencil_eval(self, q_pts, st_pts, closed=None):
        """stencil_eval (:268-298): locate at q_pts (3,N), evaluate the four
        stencil points st_pts (3,4,N) in that sub-triangle, not normalised.
        closed=True evaluates the sub-triangle barycentrics with
        split_bary_closed (same linear map, shared rounding)."""
        closed = self.closed if closed is None else closed
        bcc, tri, vs = query(self.verts, self.tris, self.loc, q_pts.T)
        if closed:
            R = inverse_rows(vs)
            bcc = np.einsum("nij,nj->ni", R, q_pts.T)
        vn, lo, hi = split_corners(vs, bcc, self.tie_fix)
        ords = SPLIT_ORDINATES[lo, hi]
        cf = np.stack([self.coeffs[:, ords[:, k], tri] for k in range(6)], axis=-2)
        out = np.empty_like(st_pts)
        for i in range(4):
            if closed:
                b = split_bary_closed(vs, R, st_pts[:, i, :].T, lo, hi)
            else:
                b = bary(vn[:, 0], vn[:, 1], vn[:, 2], st_pts[:, i, :].T)
            out[:, i, :] = _sbb(cf, b)
        return out


class CompositeOracle:
    """composite_sphere_diffeomorphism (cmm_s2/core/spherical_spline.py:340-508)."""

    def __init__(self, verts, tris, locator, vals_stack, geom=None, tie_fix=False, closed=False):
        self.verts, self.tris, self.loc = verts, tris, locator
        self.tie_fix, self.closed = tie_fix, closed
        self.geom = geom if geom is not None else ps_split(verts, tris)
        self.vals = vals_stack
        self.coeffs = np.stack([assemble(verts, tris, v, self.geom) for v in vals_stack])

    def __call__(self, q, n_c=None, record=False):
        """__call__ (:365-398): apply submaps Nc-1 ... 0; q (N,3) -> (N,3).

        With record=True also returns per-submap triangle ids (S,N) and the
        intermediate points, in application order."""
        n_c = len(self.vals) if n_c is None else n_c
        p = q.copy()
        tris, pts = [], []
        for i in reversed(range(n_c)):
            bcc, tri, vs = query(self.verts, self.tris, self.loc, p)
            out = eval_patch(self.coeffs[i], tri, bcc, vs, p, self.tie_fix, self.closed)
            nrm = np.sqrt(out[0] ** 2 + out[1] ** 2 + out[2] ** 2)
            tris.append(tri)
            pts.append(p)
            p = ((1 / nrm)[None] * out).T
        if record:
            return p, np.array(tris), pts
        return p


# ---------------------------------------------------------------- Jacobians
def patch_jacobian(coeffs, tri, bcc_big, vs, p, tie_fix=False):
    """Tangent Jacobian of one normalised submap at p (N,3): (N,3,3).

    The reference's ``eval_grad`` (cmm_s2/core/spherical_spline.py:208-265)
    refers to attributes that do not exist; this restates it from the
    working scalar ``spherical_spline.gradient`` (:73-111), ``grad_HBB``
    (:700-713) and the normalisation derivative (:247-263):
    P(x) = sum_k B_k(gamma(x)) c_k with gamma linear in x,
    J = (I - s s^T) DP (I - p p^T) / |P|, s = P/|P|."""
    vn, lo, hi = split_corners(vs, bcc_big, tie_fix)
    ords = SPLIT_ORDINATES[lo, hi]
    b = bary(vn[:, 0], vn[:, 1], vn[:, 2], p)
    eye = np.eye(3)
    # d gamma / d x: the barycentrics of the unit vectors (gradient, :89-97)
    db = np.stack([bary(vn[:, 0], vn[:, 1], vn[:, 2], np.broadcast_to(eye[j], p.shape)) for j in range(3)], 2)
    cf = np.stack([coeffs[:, ords[:, k], tri] for k in range(6)], axis=-2)       # (3,6,N)
    P = _sbb(cf, b)                                                             # (3,N)
    dp1 = 2 * cf[:, 0] * b[:, 0] + 2 * cf[:, 3] * b[:, 1] + 2 * cf[:, 5] * b[:, 2]
    dp2 = 2 * cf[:, 1] * b[:, 1] + 2 * cf[:, 3] * b[:, 0] + 2 * cf[:, 4] * b[:, 2]
    dp3 = 2 * cf[:, 2] * b[:, 2] + 2 * cf[:, 4] * b[:, 1] + 2 * cf[:, 5] * b[:, 0]
    dpg = np.stack([dp1, dp2, dp3], 2)                                          # (3,N,3) d P_c / d gamma_i
    DP = np.einsum("cni,nij->ncj", dpg, db)                                      # (N,3,3) d P_c / d x_j
    nrm = np.sqrt(P[0] ** 2 + P[1] ** 2 + P[2] ** 2)
    s = (P / nrm).T
    Ps = np.eye(3)[None] - s[:, :, None] * s[:, None, :]
    Pp = np.eye(3)[None] - p[:, :, None] * p[:, None, :]
    return np.einsum("nab,nbc,ncd->nad", Ps, DP, Pp) / nrm[:, None, None], s


def composite_jacobian(comp, q, n_c=None):
    """Chained tangent Jacobian of the composite map at q: returns (image (N,3),
    J (N,3,3)) with J = J_0(x_{S-1}) ... J_{S-1}(q)."""
    n_c = len(comp.vals) if n_c is None else n_c
    p = q.copy()
    J = np.broadcast_to(np.eye(3), (len(q), 3, 3)).copy()
    for i in reversed(range(n_c)):
        bcc, tri, vs = query(comp.verts, comp.tris, comp.loc, p)
        Ji, s = patch_jacobian(comp.coeffs[i], tri, bcc, vs, p, comp.tie_fix)
        J = np.einsum("nab,nbc->nac", Ji, J)
        p = s
    return p, J


# -------------------------------------------------------- velocity interpolant
class VelocityOracle:
    """spline_interp_velocity (cmm_s2/core/spherical_spline.py:545-655) on a
    LatLonMesh; vals (3 time levels,3,4,Nv_u)."""

    def __init__(self, mesh, vals, ts):
        self.mesh = mesh
        self.vals = vals
        self.ts = np.asarray(ts, dtype=np.float64)
        self.geom = ps_split(mesh.vertices, mesh.simplices)
        self.coeffs = np.zeros((3, 3, 19, len(mesh.simplices)))
        self.nVs = 1
        self.stepping = False

    def init_coeffs(self, i):
        self.coeffs[i] = assemble(self.mesh.vertices, self.mesh.simplices, self.vals[i], self.geom)

    def __call__(self, t, dt, q):
        """__call__ (:570-615); q (3,N) -> (3,N)."""
        bcc, tri, vs = self.mesh.query(q.T)
        outs = eval_patch(self.coeffs, tri, bcc, vs, q.T)        # (3 levels,3,N)
        if self.nVs == 3:
            t0, t1, t2 = self.ts[0], self.ts[0] + dt, self.ts[0] + 2 * dt
            l0 = (t - t1) * (t - t2) / (2 * dt ** 2)
            l1 = (t - t0) * (t - t2) / (-dt ** 2)
            l2 = (t - t0) * (t - t1) / (2 * dt ** 2)
            return l0 * outs[0] + l1 * outs[1] + l2 * outs[2]
        if self.nVs == 1:
            return outs[0]
        if self.nVs == 2:
            tau = (t - self.ts[0]) / dt
            return (1 - tau) * outs[0] + tau * outs[1]
        return outs
