"""Reference FP64 gradient of a whole barotropic run (test infrastructure).

TEST INFRASTRUCTURE ONLY, like the rest of ``oracle``: a pure-torch FP64
restatement of the reference driver euler_simulation_sphere_remapping
(cmm_s2/core/spherical_simulations.py:144-297) with the initial vorticity a
real spherical-harmonic series, assembled from the numpy oracle's pieces, so
that torch autograd on the CPU gives an independent gradient of
J = sum_x W(x) (omega_T(x) - target(x))^2 with respect to the series
coefficients.  Every stage is a torch operation on the differentiated
tensors:

* the 19 Powell-Sabin ordinates from vertex jets (assemble_coefficients,
  cmm_s2/core/spherical_spline.py:300-337), for the map and the velocity;
* map and velocity patches (:178-205, :570-615) with the closed-form
  sub-triangle barycentrics of ``oracle.spline.split_bary_closed``;
* the quadratic Lagrange velocity interpolation in time (:596-602) and the
  backward integrators with sphere projection
  (cmm_s2/core/evolution_functions.py:19-85);
* the map update: stencil foot points, the previous map evaluated in the
  sub-triangle of the vertex foot point, stencil average and differences
  (:90-142);
* the MWSS transforms of ``oracle.sht``, inv_Laplacian and project_stream
  (cmm_s2/core/spherical_harmonic_tools.py:14-105);
* the vorticity at the back-traced points (``oracle.vorticity_torch``) and
  the composition of the grid points through the submaps
  (``oracle.compose_torch``).

The piecewise choices -- containing triangles (icosahedral mesh: the
oracle's cone locator; lat-lon mesh: the reference's structured query) and
Powell-Sabin sub-triangles -- are made on the detached forward points and
held fixed, as in the library's adjoint.  The run's schedule (bootstrap with
Euler, improved Euler and a first RK4 step; remaps; velocity-level
rotation) follows the reference driver line by line.
"""
import numpy as np
import torch

from . import sht as S
from .compose_torch import composite_eval
from .evolution import identity_jets
from .geometry import ConeLocator, LatLonMesh, ps_split, query, stencil_points
from .spline import SPLIT_CORNERS, SPLIT_ORDINATES, inverse_rows
from .vorticity_torch import sampled_vorticity

T64 = torch.float64


def _t(a):
    return torch.from_numpy(np.ascontiguousarray(a))


# ------------------------------------------------------------- splines
def assemble_t(vals, tris, geom):
    """oracle.spline.assemble in torch: vals (C,4,Nv) -> coeffs (C,19,Nt)."""
    H, G, E = geom
    tv = vals[:, :, _t(tris)]                       # (C,4,Nt,3)

    def grad_ord(k, gi, corner):
        h, g = _t(H[k]), _t(G[k])
        dot = h[:, 0] * tv[0, 1:, :, corner] + h[:, 1] * tv[1, 1:, :, corner] + h[:, 2] * tv[2, 1:, :, corner]
        return (1 / g[:, gi])[None] * (dot / 2 - g[:, 0][None] * tv[:, 0, :, corner])

    o = [tv[:, 0, :, 0], tv[:, 0, :, 1], tv[:, 0, :, 2]]
    for k, gi, corner in ((0, 1, 0), (6, 1, 0), (4, 2, 0), (2, 1, 1), (7, 1, 1), (1, 2, 1),
                          (5, 1, 2), (8, 1, 2), (3, 2, 2)):
        o.append(grad_ord(k, gi, corner))
    e1, e2, e3, mid = _t(E[0]), _t(E[1]), _t(E[2]), _t(G[9])
    o.append(e1[:, 0] * o[3] + e1[:, 1] * o[8])
    o.append(e2[:, 1] * o[6] + e2[:, 2] * o[11])
    o.append(e3[:, 2] * o[9] + e3[:, 0] * o[5])
    o.append(e1[:, 0] * o[4] + e1[:, 1] * o[7])
    o.append(e2[:, 1] * o[7] + e2[:, 2] * o[10])
    o.append(e3[:, 0] * o[4] + e3[:, 2] * o[10])
    o.append(mid[:, 0] * o[4] + mid[:, 1] * o[7] + mid[:, 2] * o[10])
    return torch.stack(o, 1)


def choices(qfn, pts):
    """The piecewise choices at the points pts (N,3) (numpy): containing
    triangle by qfn (-> bcc, tri, vs), inverse vertex rows, Powell-Sabin
    sub-triangle (argmin, argmax of R p; (1, 0) at the split centre) and
    the edge/centre norms of the closed form."""
    _, tri, vs = qfn(pts)
    R = inverse_rows(vs)
    b = np.einsum("nij,nj->ni", R, pts)
    lo, hi = np.argmin(b, axis=1), np.argmax(b, axis=1)
    tie = lo == hi
    lo, hi = np.where(tie, 1, lo), np.where(tie, 0, hi)
    n = np.arange(len(pts))
    mid = 3 - lo - hi
    return dict(tri=_t(tri), R=_t(R), lo=_t(lo), hi=_t(hi), mid=_t(mid), n=_t(n),
                N4=_t(np.linalg.norm(vs.sum(1), axis=1)),
                Ne=_t(np.linalg.norm(vs[n, hi] + vs[n, mid], axis=1)),
                corn=_t(SPLIT_CORNERS[lo, hi]), ords=_t(SPLIT_ORDINATES[lo, hi]))


def patch(coeffs, ch, p):
    """Un-normalised patch values (C,N) of coeffs (C,19,Nt) at p (N,3)
    under the fixed choices ch."""
    b = torch.einsum("nij,nj->ni", ch["R"], p)
    n = ch["n"]
    gV = b[n, ch["hi"]] - b[n, ch["mid"]]
    gE = ch["Ne"] * (b[n, ch["mid"]] - b[n, ch["lo"]])
    gC = ch["N4"] * b[n, ch["lo"]]
    corn = ch["corn"]
    g = [torch.where(corn[:, k] == ch["hi"], gV, torch.where(corn[:, k] == 3, gC, gE)) for k in range(3)]
    cf = coeffs[:, ch["ords"], ch["tri"][:, None]]            # (C,N,6)
    return (g[0] ** 2 * cf[..., 0] + g[1] ** 2 * cf[..., 1] + g[2] ** 2 * cf[..., 2]
            + 2 * g[1] * g[0] * cf[..., 3] + 2 * g[2] * g[1] * cf[..., 4] + 2 * g[2] * g[0] * cf[..., 5])


def _proj(x):
    """div_norm (cmm_s2/core/evolution_functions.py:82-85) on rows."""
    return x / torch.sqrt((x * x).sum(1, keepdim=True))


# ------------------------------------------------------------- transforms
class TorchSHT:
    """oracle.sht.MWSS and the coefficient-space operators in torch."""

    def __init__(self, L):
        self.L = L
        m = S.MWSS(L)
        self.P = _t(m.P).to(torch.complex128)                # (L,L,L+1) [l,m,t]
        self.Pf = _t(m.Pf).to(torch.complex128)              # (L,L,2L+1)
        self.w = _t(m.w).to(torch.complex128)
        self.dinv = _t(S.inverse_laplacian_diag(L))
        lp, lm, lz = S.ladder_operators(L)
        self.lp, self.lm, self.lz = _t(lp), _t(lm), _t(lz)
        ls, cs, src, conj_sign = [], [], [], []
        for l in range(L):                                    # shifted layout from the m >= 0 half
            for mm in range(-l, l + 1):
                ls.append(l)
                cs.append(l + mm)
                src.append(l * L + abs(mm))
                conj_sign.append(0 if mm >= 0 else (-1) ** mm)
        self.sh_l, self.sh_c = _t(np.array(ls)), _t(np.array(cs))
        self.sh_src, self.sh_sign = _t(np.array(src)), _t(np.array(conj_sign, dtype=np.float64))
        hl, hm = np.nonzero(np.tril(np.ones((L, L), dtype=bool)))
        self.h_l, self.h_m = _t(hl), _t(hm)

    def forward(self, f):
        """real samples (L+1, 2L) -> (L,L) complex [l, m >= 0]."""
        L = self.L
        Fm = torch.fft.rfft(f, dim=1)[:, :L] * (np.pi / L)
        sign = _t((-1.0) ** np.arange(L)).to(torch.complex128)
        G = torch.cat([Fm, sign * torch.flip(Fm[1:L], dims=[0])], 0)
        Gh = torch.fft.fft(G, dim=0) / (2 * L)
        z = torch.zeros((2 * L - 1, L), dtype=torch.complex128)
        H = torch.cat([Gh[:L], Gh[L:L + 1] / 2, z, Gh[L:L + 1] / 2, Gh[L + 1:]], 0)
        fine = torch.fft.ifft(H, dim=0)[:2 * L + 1] * (4 * L)
        return torch.einsum("jm,lmj,j->lm", fine, self.Pf, self.w)

    def inverse(self, alm):
        """(L,L) complex [l, m >= 0] -> real samples (L+1, 2L)."""
        L = self.L
        F = torch.einsum("lm,lmt->tm", alm, self.P)
        c = torch.cat([F, torch.zeros((L + 1, 1), dtype=torch.complex128)], 1)
        return torch.fft.irfft(c, n=2 * L, dim=1) * (2 * L)

    def shifted(self, alm):
        """(L,L) [l, m >= 0] -> coeff_array layout (L, 2L+1), column l + m,
        a_{l,-m} = (-1)^m conj(a_lm)."""
        v = alm.reshape(-1)[self.sh_src]
        v = torch.where(self.sh_sign == 0, v, self.sh_sign * torch.conj(v))
        out = torch.zeros((self.L, 2 * self.L + 1), dtype=torch.complex128)
        return out.index_put((self.sh_l, self.sh_c), v)

    def half(self, c):
        """coeff_array layout -> (L,L) [l, m >= 0] (columns l + m)."""
        out = torch.zeros((self.L, self.L), dtype=torch.complex128)
        return out.index_put((self.h_l, self.h_m), c[self.h_l, self.h_l + self.h_m])

    def angular_momentum(self, a):
        """i(L_x, L_y, L_z) (cmm_s2/core/spherical_harmonic_tools.py:49-62)."""
        z = torch.zeros((self.L, 1), dtype=torch.complex128)
        up = self.lp * torch.cat([z, a[:, :-1]], 1)
        dn = self.lm * torch.cat([a[:, 1:], z], 1)
        ox = (up + dn) / 2
        oy = 1j * (dn - up) / 2
        return [1j * ox, 1j * oy, 1j * (self.lz * a)]


# ---------------------------------------------------------------- the run
class BVETorch:
    """The reference driver in torch for the gradient check; same arguments
    as the library's BVEGradient (level mesh, band-limit L, Nt steps over
    [0, T], remap every n_maps steps)."""

    def __init__(self, verts, tris, L, Nt, T, rot_rate=2 * np.pi, n_maps=10, eps=1e-5):
        self.verts, self.tris = verts, tris
        self.loc = ConeLocator(verts, tris)
        self.geom = ps_split(verts, tris)
        tan, s_pts = stencil_points(verts, eps)
        self.tan, self.s_pts, self.eps = _t(tan), _t(s_pts), eps
        self.mu = LatLonMesh(L)
        self.geom_u = ps_split(self.mu.vertices, self.mu.simplices)
        self.sht = TorchSHT(L)
        self.L, self.Nt, self.rot = L, Nt, rot_rate
        self.tspan = np.linspace(0, T, Nt, endpoint=False)
        self.dt = float(self.tspan[1] - self.tspan[0])
        ns = [i for i in range(1, Nt) if i % n_maps == 0]
        self.ns = ns + [Nt]
        g = self.mu.grid_points
        self.X = _t(np.stack([c.reshape(-1) for c in g], 1))     # (Q,3) sample points
        self.cos_grid = self.X[:, 2].clone()
        theta = self.mu.theta
        w = np.sin(theta) * (np.pi / L) ** 2
        self.W = _t(np.repeat(w[:, None], 2 * L, 1))
        self.id_jets = _t(identity_jets(verts))

    # -- velocity
    def velocity_jets(self, psi):
        """project_stream's spatial part (oracle.sht.velocity_jets)."""
        sh, L = self.sht, self.L
        X = self.X.T.reshape(3, L + 1, 2 * L)

        def put(f):
            return torch.cat([f[0, :1], f[1:-1].reshape(-1), f[-1, :1]])

        u = sh.angular_momentum(psi)
        rows = [[None] * 4 for _ in range(3)]
        for i in range(3):
            rows[i][0] = put(sh.inverse(sh.half(u[i])))
            G = [sh.inverse(sh.half(gk)) for gk in sh.angular_momentum(u[i])]
            cr = [G[1] * X[2] - G[2] * X[1], G[2] * X[0] - G[0] * X[2], G[0] * X[1] - G[1] * X[0]]
            sc = (cr[0] * X[0] + cr[1] * X[1] + cr[2] * X[2]) / torch.sqrt(X[0] ** 2 + X[1] ** 2 + X[2] ** 2)
            for c in range(3):
                rows[c][1 + i] = put(cr[c] - sc * X[c])
        return torch.stack([torch.stack(r) for r in rows])      # (3,4,Nv_u)

    def project(self, Xs, sh, rot):
        """vorticity at the back-traced sample points -> velocity records
        (3,19,Nt_u) and the vorticity (L+1, 2L)."""
        L = self.L
        om = sampled_vorticity(sh, Xs, rot, self.cos_grid).reshape(L + 1, 2 * L)
        alm = self.sht.forward(om)
        psi = self.sht.shifted(alm) * self.sht.dinv[:, None]
        return assemble_t(self.velocity_jets(psi), self.mu.simplices, self.geom_u), om

    def vel(self, levels, nvs, ts0, t, x):
        """spline_interp_velocity.__call__ (:570-615) at time t, x (N,3)."""
        ch = choices(lambda q: self.mu.query(q), x.detach().numpy())
        outs = [patch(c, ch, x) for c in levels[:nvs]]
        dt = self.dt
        if nvs == 1:
            v = outs[0]
        elif nvs == 2:
            tau = (t - ts0) / dt
            v = (1 - tau) * outs[0] + tau * outs[1]
        else:
            t0, t1, t2 = ts0, ts0 + dt, ts0 + 2 * dt
            l0 = (t - t1) * (t - t2) / (2 * dt ** 2)
            l1 = (t - t0) * (t - t2) / (-dt ** 2)
            l2 = (t - t0) * (t - t1) / (2 * dt ** 2)
            v = l0 * outs[0] + l1 * outs[1] + l2 * outs[2]
        return v.T

    def integrate(self, scheme, t, x, V):
        dt = self.dt
        if scheme == "euler":
            return _proj(x - dt * V(t, x))
        if scheme == "ieuler":
            v1 = V(t, x)
            s1 = _proj(x - dt * v1)
            v2 = V(t + dt, s1)
            return _proj(x - (dt / 2) * (v1 + v2))
        v1 = V(t + dt, x)
        s1 = _proj(x - dt * v1 / 2)
        v2 = V(t + dt / 2, s1)
        s2 = _proj(x - (dt / 2) * v2)
        v3 = V(t + 0.5 * dt, s2)
        s3 = _proj(x - dt * v3)
        v4 = V(t, s3)
        return _proj(x - (dt / 6) * (v1 + 2 * v2 + 2 * v3 + v4))

    def advect(self, prev, levels, nvs, ts0, scheme, t):
        """advect_project_sphere (cmm_s2/core/evolution_functions.py:117-142):
        previous map coefficients (None = identity) -> new coefficients."""
        nv = len(self.verts)

        def V(tt, x):
            return self.vel(levels, nvs, ts0, tt, x)

        yn = self.integrate(scheme, t, _t(self.verts), V)
        sp = self.s_pts.permute(1, 2, 0).reshape(4 * nv, 3)
        sn = self.integrate(scheme, t, sp, V).reshape(4, nv, 3)
        if prev is not None:
            ch = choices(lambda q: query(self.verts, self.tris, self.loc, q), yn.detach().numpy())
            sn = torch.stack([patch(prev, ch, sn[i]) for i in range(4)], 1)     # (3,4,Nv)
        else:
            sn = sn.permute(2, 0, 1)
        m = (sn[:, 0] + sn[:, 1] + sn[:, 2] + sn[:, 3]) / 4
        val = m / torch.sqrt((m * m).sum(0, keepdim=True))
        d1 = (sn[:, 1] - sn[:, 0] + sn[:, 3] - sn[:, 2]) / (4 * self.eps)
        d2 = (sn[:, 2] - sn[:, 0] + sn[:, 3] - sn[:, 1]) / (4 * self.eps)
        grads = [(d1[k][:, None] * self.tan[0] + d2[k][:, None] * self.tan[1]).T for k in range(3)]
        jets = torch.stack([val, *grads], 1)                      # (3,4,Nv): [j, 1+k] = d_j f_k
        return assemble_t(jets, self.tris, self.geom)

    def sample(self, maps):
        return composite_eval(maps, self.X, self.verts, self.tris, self.loc)

    def omega_T(self, sh):
        """The final vorticity (L+1, 2L) of the run from the real series sh."""
        dt, ts0 = self.dt, float(self.tspan[0])
        v0, _ = self.project(self.X, sh, 0.0)
        c = self.advect(None, [v0], 1, ts0, "euler", 0.0)
        v1, _ = self.project(self.sample([c]), sh, self.rot)
        c = self.advect(None, [v0, v1], 2, ts0, "ieuler", 0.0)
        v1, _ = self.project(self.sample([c]), sh, self.rot)
        c = self.advect(c, [v0, v1], 2, ts0, "rk4", dt)
        v2, om = self.project(self.sample([c]), sh, self.rot)
        vel, stack, identity, count = [v0, v1, v2], [], False, 2
        for k in range(2, self.Nt):
            t = float(self.tspan[k])
            c = self.advect(None if identity else c, vel, 3, ts0, "rk4", t)
            vn, om = self.project(self.sample(stack + [c]), sh, self.rot)
            vel = [vel[1], vel[2], vn]
            ts0 += dt
            count += 1
            identity = False
            if count in self.ns:
                stack.append(c)
                identity = True
        return om

    def gradient(self, sh, target):
        """(J, dJ/dsh) by torch autograd: sh (lmax+1, 2 lmax+1), target
        (L+1, 2L), both numpy or torch."""
        a = torch.as_tensor(np.asarray(sh), dtype=T64).clone().requires_grad_(True)
        tg = torch.as_tensor(np.asarray(target), dtype=T64)
        J = (self.W * (self.omega_T(a) - tg) ** 2).sum()
        J.backward()
        return float(J.detach()), a.grad.detach().numpy()
