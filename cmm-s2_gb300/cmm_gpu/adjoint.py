"""Hand-written adjoints of the CMM hot path behind torch.autograd.Function.

Each Function's forward is the library's forward call and its backward the
library's reverse-mode twin (include/cmm_gpu.h, "adjoints"), so a barotropic
run expressed with these Functions is differentiated by torch's autograd
engine without torch ever differentiating the arithmetic itself.
``BVEGradient`` builds the whole run that way (with each remap interval
checkpointed and recomputed in the backward pass) and returns the gradient
of J = sum_x W(x) (omega_T(x) - omega_target(x))^2 over the MWSS grid with
respect to the initial real spherical-harmonic coefficients.

No counterpart in the reference (it has no derivatives).
"""
import ctypes

import numpy as np
import torch
from torch.utils.checkpoint import checkpoint

from . import native
from .meshgen import icosahedral_mesh, identity_jets, latlon_mesh_arrays, stencil_frames


def _s(dev):
    return native._stream(dev)


# ------------------------------------------------------ SH coefficient maps
def real_to_complex(a):
    """Real series (lmax+1, 2 lmax+1) (column l+m; m > 0 sqrt2 cos, m < 0
    sqrt2 sin) -> complex half layout c[l, m] (m >= 0) of the same field."""
    lmax = a.shape[0] - 1
    c = np.zeros((lmax + 1, lmax + 1), dtype=complex)
    for l in range(lmax + 1):
        c[l, 0] = a[l, l]
        for m in range(1, l + 1):
            c[l, m] = (a[l, l + m] - 1j * a[l, l - m]) / np.sqrt(2)
    return c


def complex_to_real(c):
    lmax = c.shape[0] - 1
    a = np.zeros((lmax + 1, 2 * lmax + 1))
    for l in range(lmax + 1):
        a[l, l] = c[l, 0].real
        for m in range(1, l + 1):
            a[l, l + m] = np.sqrt(2) * c[l, m].real
            a[l, l - m] = -np.sqrt(2) * c[l, m].imag
    return a


def il_series(a):
    """The three real series iL_x f, iL_y f, iL_z f of the real series f
    (angular-momentum operators with L+ Y_lm = sqrt((l-m)(l+m+1)) Y_l,m+1,
    a_{l,-1} = -conj(a_{l,1}) for a real field); the tangent gradient of f
    at a unit point x is -x cross (iL f)(x).  Returns (3, lmax+1, 2 lmax+1)."""
    c = real_to_complex(np.asarray(a, dtype=np.float64))
    lmax = c.shape[0] - 1
    out = [np.zeros_like(c) for _ in range(3)]
    for l in range(lmax + 1):
        ll = l * (l + 1.0)
        for m in range(0, l + 1):
            am1 = -np.conj(c[l, 1]) if m == 0 and l >= 1 else (c[l, m - 1] if m >= 1 else 0.0)
            ap1 = c[l, m + 1] if m + 1 <= l else 0.0
            up = np.sqrt(ll - m * (m - 1.0)) * am1
            dn = np.sqrt(ll - m * (m + 1.0)) * ap1
            out[0][l, m] = 1j * (up + dn) / 2
            out[1][l, m] = (up - dn) / 2
            out[2][l, m] = 1j * m * c[l, m]
    return np.stack([complex_to_real(o) for o in out])


# ------------------------------------------------------- autograd Functions
class Assemble(torch.autograd.Function):
    """jets (3,4,Nv) -> coefficient records (Nt,64), FP64 (cmm_assemble)."""

    @staticmethod
    def forward(ctx, jets, mesh):
        ctx.mesh = mesh
        return mesh.assemble(jets.detach().contiguous())

    @staticmethod
    def backward(ctx, gc):
        mesh = ctx.mesh
        gc = gc.contiguous()
        gj = torch.zeros((3, 4, mesh.nv), dtype=torch.float64, device=gc.device)
        native.check(native.lib.cmm_assemble_bwd(mesh.h, native._ptr(gc), native._ptr(gj), _s(gc.device)),
                     "cmm_assemble_bwd")
        return gj, None


class Compose(torch.autograd.Function):
    """Points q (n,3) through the submaps (coefficient records, submap 0
    applied last) -> (n,3) (cmm_compose without Jacobians)."""

    @staticmethod
    def forward(ctx, q, mesh, *coeffs):
        ctx.mesh = mesh
        ctx.save_for_backward(q, *coeffs)
        out, _, _, _ = mesh.compose([c.detach() for c in coeffs], q.detach())
        return out

    @staticmethod
    def backward(ctx, gout):
        q, *coeffs = ctx.saved_tensors
        mesh = ctx.mesh
        dev = q.device
        n, S = q.shape[0], len(coeffs)
        gcs = [torch.zeros_like(c) for c in coeffs]
        gq = torch.zeros_like(q) if ctx.needs_input_grad[0] else None
        work = torch.empty(3 * S * n, dtype=torch.float64, device=dev)
        ca = (ctypes.c_void_p * S)(*[c.data_ptr() for c in coeffs])
        ga = (ctypes.c_void_p * S)(*[g.data_ptr() for g in gcs])
        native.check(native.lib.cmm_compose_bwd(mesh.h, ca, S, native._ptr(q), n,
                                                native._ptr(gout.contiguous()), ga, native._ptr(gq),
                                                native._ptr(work), _s(dev)), "cmm_compose_bwd")
        return (gq, None, *gcs)


class Vorticity(torch.autograd.Function):
    """omega (L+1, 2L) at the back-traced points X (Q,3) from the real
    series sh and the planetary term (cmm_vorticity_eval, kind NONE)."""

    @staticmethod
    def forward(ctx, X, sh, vm, rot):
        ctx.vm, ctx.rot = vm, rot
        ctx.save_for_backward(X, sh)
        return vm.vorticity(native.VORT_NONE, [], X.detach(), rot, sh=sh.detach())

    @staticmethod
    def backward(ctx, gw):
        X, sh = ctx.saved_tensors
        vm = ctx.vm
        lmax = sh.shape[0] - 1
        dsh = torch.from_numpy(il_series(sh.detach().cpu().numpy())).to(X.device)
        gX = torch.zeros_like(X)
        gsh = torch.zeros_like(sh)
        native.check(native.lib.cmm_vorticity_bwd(vm.h, native._ptr(dsh), lmax, ctx.rot, native._ptr(X),
                                                  native._ptr(gw.contiguous()), native._ptr(gX),
                                                  native._ptr(gsh), _s(X.device)), "cmm_vorticity_bwd")
        return gX, gsh, None, None


class Velocity(torch.autograd.Function):
    """omega (L+1, 2L) -> velocity jets (3,4,Nv_u) (cmm_sht_velocity, FP64)."""

    @staticmethod
    def forward(ctx, omega, sht, vm):
        ctx.sht, ctx.vm = sht, vm
        return sht.velocity(vm, omega.detach().contiguous())

    @staticmethod
    def backward(ctx, gj):
        sht, vm = ctx.sht, ctx.vm
        gw = torch.empty((sht.L + 1, 2 * sht.L), dtype=torch.float64, device=gj.device)
        native.check(native.lib.cmm_sht_velocity_bwd(sht.h, vm.h, native._ptr(gj.contiguous()),
                                                     native._ptr(gw), _s(gj.device)), "cmm_sht_velocity_bwd")
        return gw, None, None


class AdvectProject(torch.autograd.Function):
    """Map update (cmm_advect_project): previous map records (empty tensor =
    identity) and nvs velocity levels -> new jets (3,4,Nv)."""

    @staticmethod
    def forward(ctx, prev, v0, v1, v2, mesh, vm, nvs, ts0, scheme, t, dt, s_pts, tan):
        ctx.args = (mesh, vm, nvs, ts0, scheme, t, dt, s_pts, tan)
        ctx.has_prev = prev.numel() > 0
        ctx.save_for_backward(prev, v0, v1, v2)
        vel = [v.detach() for v in (v0, v1, v2)[:nvs]]
        jets, _ = mesh.advect_project(vm, vel, ts0, scheme, t, dt, s_pts, tan,
                                      prev.detach() if ctx.has_prev else None)
        return jets

    @staticmethod
    def backward(ctx, gj):
        prev, v0, v1, v2 = ctx.saved_tensors
        mesh, vm, nvs, ts0, scheme, t, dt, s_pts, tan = ctx.args
        dev = gj.device
        vel = (v0, v1, v2)[:nvs]
        gvel = [torch.zeros_like(v) for v in vel]
        gprev = torch.zeros_like(prev) if ctx.has_prev else None
        nw = native.lib.cmm_advect_workspace(mesh.h) + 12 * mesh.nv
        work = torch.empty(nw, dtype=torch.float64, device=dev)
        va = (ctypes.c_void_p * nvs)(*[v.data_ptr() for v in vel])
        ga = (ctypes.c_void_p * nvs)(*[g.data_ptr() for g in gvel])
        native.check(native.lib.cmm_advect_project_bwd(
            mesh.h, vm.h, va, nvs, ts0, scheme, t, dt, native._ptr(s_pts), native._ptr(tan),
            native._ptr(prev) if ctx.has_prev else None, 1e-5, native._ptr(gj.contiguous()), ga,
            native._ptr(gprev), native._ptr(work), _s(dev)), "cmm_advect_project_bwd")
        out = [gprev] + gvel + [None] * (3 - nvs)
        # a slot passed twice (bootstrap) collects the sum of its cotangents
        return (*out, None, None, None, None, None, None, None, None, None)


# ----------------------------------------------------- the whole-run gradient
class BVEGradient:
    """The barotropic run of euler_simulation_sphere_remapping
    (cmm_s2/core/spherical_simulations.py:144-297; FP64 form, initial
    vorticity a real SH series) expressed with the Functions above, each
    remap interval under torch.utils.checkpoint (its forward recomputed in
    the backward pass), so that J(sh) = sum_x W(x) (omega_T(x) -
    target(x))^2 and dJ/dsh come from one forward and one backward pass.
    W = sin(theta) (pi/L)^2 on the MWSS grid."""

    def __init__(self, level, L, Nt, T, rot_rate=2 * np.pi, n_maps=10, device=None, checkpoint_steps=None):
        self.device = torch.device("cuda", torch.cuda.current_device() if device is None else device)
        dev = self.device
        verts, tris = icosahedral_mesh(level)
        self.mesh = native.Mesh(verts, tris, level, device=dev.index)
        theta, phi, grid, vverts = latlon_mesh_arrays(L)
        self.vm = native.VelMesh(L, theta, phi, grid, vverts, device=dev.index)
        self.sht = native.Sht(L, device=dev.index)
        tan, s_pts = stencil_frames(verts)
        self.tan = torch.from_numpy(np.ascontiguousarray(tan)).to(dev)
        self.s_pts = torch.from_numpy(np.ascontiguousarray(s_pts)).to(dev)
        self.sample = torch.from_numpy(np.ascontiguousarray(np.stack([g.reshape(-1) for g in grid], 1))).to(dev)
        self.L, self.Nt, self.rot, self.n_maps = L, Nt, rot_rate, n_maps
        self.tspan = np.linspace(0, T, Nt, endpoint=False)
        self.dt = float(self.tspan[1] - self.tspan[0])
        ns = [i for i in range(1, Nt) if i % n_maps == 0]
        self.ns = ns + [Nt]
        self.block = checkpoint_steps or n_maps
        w = np.sin(theta) * (np.pi / L) ** 2
        self.W = torch.from_numpy(np.repeat(w[:, None], 2 * L, 1)).to(dev)
        self.empty = torch.empty(0, dtype=torch.float64, device=dev)

    # pieces
    def _project(self, X, sh, rot):
        om = Vorticity.apply(X, sh, self.vm, rot)
        return Assemble.apply(Velocity.apply(om, self.sht, self.vm), self.vm), om

    def _advect(self, prev, vel, nvs, ts0, scheme, t):
        v = list(vel) + [vel[-1]] * (3 - len(vel))
        jets = AdvectProject.apply(self.empty if prev is None else prev, v[0], v[1], v[2], self.mesh, self.vm,
                                   nvs, ts0, scheme, t, self.dt, self.s_pts, self.tan)
        return Assemble.apply(jets, self.mesh)

    def _sample(self, maps):
        return Compose.apply(self.sample, self.mesh, *maps)

    def omega_T(self, sh):
        """Vorticity (L+1, 2L) on the grid at the end of the run."""
        dt, ts0 = self.dt, float(self.tspan[0])
        E, IE, RK = native.EULER, native.IMPROVED_EULER, native.RK4
        # bootstrap (spherical_simulations.py:216-261)
        v0, _ = self._project(self.sample, sh, 0.0)
        c = self._advect(None, [v0], 1, ts0, E, 0.0)
        v1, _ = self._project(self._sample([c]), sh, self.rot)
        c = self._advect(None, [v0, v1], 2, ts0, IE, 0.0)
        v1, _ = self._project(self._sample([c]), sh, self.rot)
        c = self._advect(c, [v0, v1], 2, ts0, RK, dt)
        v2, om = self._project(self._sample([c]), sh, self.rot)
        state = dict(c=c, vel=[v0, v1, v2], stack=[], identity=False, count=2, ts0=ts0, k=2, om=om)
        while state["count"] < self.Nt:
            nsteps = min(self.block, self.Nt - state["count"])
            state = self._run_block(state, sh, nsteps)
        return state["om"]

    def _steps(self, nsteps, k0, count0, ts00, identity0, nstack, sh, c, v0, v1, v2, *stack):
        """nsteps main-loop steps (spherical_simulations.py:263-294) as a
        pure function of tensors (for checkpointing)."""
        vel, stack, identity, count, ts0 = [v0, v1, v2], list(stack), identity0, count0, ts00
        om = None
        for j in range(nsteps):
            t = float(self.tspan[k0 + j])
            c = self._advect(None if identity else c, vel, 3, ts0, native.RK4, t)
            X = self._sample(stack + [c])
            vn, om = self._project(X, sh, self.rot)
            vel = [vel[1], vel[2], vn]
            ts0 += self.dt
            count += 1
            identity = False
            if count in self.ns:
                stack.append(c)
                identity = True
        return (c, *vel, om, *stack[nstack:])

    def _run_block(self, st, sh, nsteps):
        ns_before = len(st["stack"])
        args = (nsteps, st["k"], st["count"], st["ts0"], st["identity"], ns_before, sh, st["c"], *st["vel"],
                *st["stack"])
        out = checkpoint(self._steps, *args, use_reentrant=False)
        c, v0, v1, v2, om, *new = out
        count = st["count"] + nsteps
        ts0 = st["ts0"]
        identity = False
        for j in range(nsteps):
            ts0 += self.dt
            identity = (st["count"] + j + 1) in self.ns
        return dict(c=c, vel=[v0, v1, v2], stack=st["stack"] + list(new), identity=identity, count=count,
                    ts0=ts0, k=st["k"] + nsteps, om=om)

    def misfit(self, sh, target):
        om = self.omega_T(sh)
        return (self.W * (om - target) ** 2).sum()

    def gradient(self, sh, target):
        """(J, dJ/dsh) by one forward and one backward pass."""
        a = sh.detach().clone().requires_grad_(True)
        J = self.misfit(a, target)
        J.backward()
        return float(J.detach()), a.grad.detach()
