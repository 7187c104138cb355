"""Barotropic vorticity driver with remapping (oracle restatement of
euler_simulation_sphere_remapping, cmm_s2/core/spherical_simulations.py:144-297)."""
import numpy as np
from .geometry import LatLonMesh, cart2sphere, sphere2cart, ps_split, stencil_points
from .spline import MapOracle, CompositeOracle, VelocityOracle, assemble
from .evolution import (euler_back, improved_euler_back, rk4_back, advect_project, identity_jets)
from . import sht as S


class BVEOracle:
    """State and step loop of the reference driver.

    vorticity: callable (phi, theta) -> omega0 on arrays of angles."""

    def __init__(self, verts, tris, locator, L, Nt, T, vorticity, rot_rate=2 * np.pi, n_maps=10,
                 closed=False, tie_fix=False):
        """closed/tie_fix: evaluation options of MapOracle (see
        oracle.spline.split_bary_closed and split_corners)."""
        self.verts, self.tris, self.loc = verts, tris, locator
        self.closed, self.tie_fix = closed, tie_fix
        self.L, self.Nt, self.T = L, Nt, T
        self.vort, self.rot = vorticity, rot_rate
        ns = [i for i in range(1, Nt) if i % n_maps == 0]
        ns.append(Nt)
        self.ns = ns
        self.geom = ps_split(verts, tris)
        self.tan, self.s_pts = stencil_points(verts)
        self.id_jets = identity_jets(verts)
        self.stack = np.zeros((len(ns), 3, 4, len(verts)))
        self.stack[0] = self.id_jets
        self.Nc = 0
        tspan = np.linspace(0, T, Nt, endpoint=False)
        self.tspan, self.dt = tspan, tspan[1] - tspan[0]
        self.mesh_u = LatLonMesh(L)
        self.U = VelocityOracle(self.mesh_u, np.zeros((3, 3, 4, len(self.mesh_u.vertices))), tspan[0:3])
        self.sht = S.MWSS(L)
        self.dinv = S.inverse_laplacian_diag(L)
        self.lp, self.lm, self.lz = S.ladder_operators(L)
        Phi, The = np.meshgrid(self.mesh_u.phi, self.mesh_u.theta)
        self.Phi, self.The = Phi, The
        sp = sphere2cart(Phi, The)
        self.sample_pts = np.array([sp[0].reshape(-1), sp[1].reshape(-1), sp[2].reshape(-1)]).T
        self.grid_points = sp

    # ------------------------------------------------------------------
    def _map(self, jets):
        return MapOracle(self.verts, self.tris, self.loc, jets, self.geom, self.tie_fix, self.closed)

    def _vorticity_at(self, X):
        """omega at the back-traced grid points X (3,Q) (:269-272)."""
        L = self.L
        ang = cart2sphere(X)
        ph, th = ang[0].reshape(L + 1, 2 * L), ang[1].reshape(L + 1, 2 * L)
        return self.vort(ph, th) + 2 * self.rot * np.cos(th) - 2 * self.rot * np.cos(self.The)

    def _project(self, omega, n):
        """inv_Laplacian + project_stream into velocity slot n (:66-105)."""
        psi = S.inv_laplacian(omega, self.sht, self.dinv)
        if self.U.stepping:
            self.U.coeffs[0:2] = self.U.coeffs[1:3].copy()
            self.U.vals[0:2] = self.U.vals[1:3].copy()
        self.U.vals[n] = S.velocity_jets(psi, self.sht, self.grid_points, self.lp, self.lm, self.lz)
        self.U.init_coeffs(n)
        return psi

    def _advect(self, prev_jets, integ, t, identity):
        prev = None if identity else self._map(prev_jets)
        return advect_project(prev, integ, t, self.dt, self.U, self.verts, self.s_pts, self.tan, identity)

    def composite(self):
        return CompositeOracle(self.verts, self.tris, self.loc, self.stack[:self.Nc], self.geom,
                               self.tie_fix, self.closed)

    def sample_grid(self, jets):
        """submaps(curr_map(sample_pts)) (:268), (3,Q)."""
        cur = self._map(jets)(self.sample_pts)
        if self.Nc == 0:
            return cur
        return self.composite()(cur.T).T

    # ------------------------------------------------------------------
    def bootstrap(self):
        """:216-261"""
        dt = self.dt
        omega0 = self.vort(self.Phi, self.The)
        self._project(omega0, 0)
        j0 = self._advect(None, euler_back, 0.0, True)
        self._project(self._vorticity_at(self._map(j0)(self.sample_pts)), 1)
        self.U.nVs = 2
        j1 = self._advect(None, improved_euler_back, 0.0, True)
        self._project(self._vorticity_at(self._map(j1)(self.sample_pts)), 1)
        j2 = self._advect(j1, rk4_back, dt, False)
        om2 = self._vorticity_at(self._map(j2)(self.sample_pts))
        self.U.nVs = 3
        self._project(om2, 2)
        self.jets = j2
        self.U.stepping = True
        self.identity = False
        self.count = 2
        self.step_index = 2

    def step(self):
        """One pass of the main loop body (:263-294)."""
        t = self.tspan[self.step_index]
        self.jets = self._advect(self.jets, rk4_back, t, self.identity)
        X = self.sample_grid(self.jets)
        omega = self._vorticity_at(X)
        self._project(omega, 2)
        self.U.ts = self.U.ts + self.dt
        self.count += 1
        self.identity = False
        if self.count in self.ns:
            idx = self.ns.index(self.count)
            self.Nc = idx + 1
            self.stack[idx] = self.jets
            self.jets = self.id_jets.copy()
            self.identity = True
        self.step_index += 1
        self.last_omega = omega
        return omega

    def run(self, nsteps=None):
        self.bootstrap()
        n = self.Nt - 2 if nsteps is None else nsteps
        for _ in range(n):
            self.step()
        return self
