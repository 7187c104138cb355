"""Barotropic vorticity equation on the rotating sphere with the
characteristic mapping method, stepped on the GPU through libcmmgpu.so.

``BVESolver`` holds the whole state on the device and reproduces the
reference driver euler_simulation_sphere_remapping
(cmm_s2/core/spherical_simulations.py:144-297) step for step: the
Euler / improved-Euler / RK4 bootstrap (:216-261), then per step the RK4
map update, the evaluation of submaps o current map at the MWSS sample
points, the vorticity there, its inversion to velocity jets and the remap
every n_maps steps.
"""
import ctypes
import math

import numpy as np
import torch

from . import native
from .meshgen import identity_jets, latlon_mesh_arrays, stencil_frames

_FIELDS = {
    "rossby_wave": native.VORT_ROSSBY_HAURWITZ,
    "zonal_jet": native.VORT_ZONAL_JET,
    "perturbed_zonal_jet": native.VORT_PERTURBED_JET,
    "multi_jet": native.VORT_MULTI_JET,
    "gaussian_vortex": native.VORT_GAUSSIAN_VORTEX,
    "gaussian_zonal_jets": native.VORT_GAUSSIAN_JETS,
    "perturbed_rossby_wave": native.VORT_PERTURBED_RH,
}


class Vorticity:
    """Initial vorticity evaluated on the device: a built-in field of
    cmm_s2/core/dynamical_fields.py (by name), plus optionally a real
    spherical-harmonic series (coefficients (lmax+1, 2lmax+1), column l+m)
    evaluated either pointwise (`sh`) or through its scalar Powell-Sabin
    spline on the velocity mesh (`spline_sh`, the reference's
    project_onto_S12 route, cmm_s2/core/spherical_harmonic_tools.py:108-142;
    ~150 operations per point instead of O(lmax^2))."""

    def __init__(self, field=None, params=(), sh=None, spline_sh=None):
        self.kind = _FIELDS[field] if field is not None else native.VORT_NONE
        self.params = np.asarray(params, dtype=np.float64)
        self.sh = None if sh is None else np.ascontiguousarray(sh, dtype=np.float64)
        self.spline_sh = None if spline_sh is None else np.ascontiguousarray(spline_sh, dtype=np.float64)

    @classmethod
    def from_reference(cls, f):
        """Accept a reference field function (or its name)."""
        if isinstance(f, Vorticity):
            return f
        name = f if isinstance(f, str) else getattr(f, "__name__", None)
        if name not in _FIELDS:
            raise ValueError(f"no device implementation of vorticity field {name!r}")
        return cls(name, (0.0,) if name == "rossby_wave" else ())


class BVESolver:
    def __init__(self, verts, tris, level, L, Nt, T, vorticity, rot_rate=2 * np.pi, n_maps=10,
                 device=None, precision="fp64", resources=None, fp64_tables=None, forms=True):
        """verts, tris: the icosahedral mesh of `level` (reference row order);
        with `resources` (ensemble.SharedResources) they may be None and the
        mesh, stencil frames, velocity mesh, sample points and split-BF16
        tables are taken from (and shared through) it.  fp64_tables: the
        FP64 Legendre stages from Pbar tables (True), from the recurrence
        (False) or by band-limit (None: tables for L <= 512).  forms: every
        remapped submap also gets its map-form records (cmm_assemble_forms,
        the patches as quadratic forms; 0.9 KB per triangle), through which
        the sample points cross the stack at every step (the current map
        stays on its coefficient records)."""
        self.device = torch.device("cuda", torch.cuda.current_device() if device is None else device)
        dev = self.device
        if precision not in ("fp64", "split_bf16"):
            raise ValueError("precision must be 'fp64' or 'split_bf16'")
        split = precision == "split_bf16"
        self.vort = Vorticity.from_reference(vorticity)
        self.sh = None if self.vort.sh is None else torch.from_numpy(self.vort.sh).to(dev)
        self.L, self.Nt, self.T, self.rot, self.n_maps = L, Nt, T, rot_rate, n_maps
        self.level = level
        if resources is not None:
            verts, tris, self.mesh = resources.mesh(level)
            self.vm = resources.velmesh(L, split)[0]
            self.tan, self.s_pts, self.id_jets = resources.frames(level)
            self.sample_pts = resources.sample_pts(L)
        else:
            self.mesh = native.Mesh(verts, tris, level, device=dev.index)
            theta, phi, grid, vverts = latlon_mesh_arrays(L)
            self.vm = native.VelMesh(L, theta, phi, grid, vverts, device=dev.index)
            if split:
                # the mixed form keeps its velocity records in FP32
                self.vm.set_records(native.VelMesh.REC_MIXED)
            tan, s_pts = stencil_frames(verts)
            self.tan = torch.from_numpy(np.ascontiguousarray(tan)).to(dev)
            self.s_pts = torch.from_numpy(np.ascontiguousarray(s_pts)).to(dev)
            self.id_jets = torch.from_numpy(identity_jets(verts)).to(dev)
            self.sample_pts = torch.from_numpy(
                np.ascontiguousarray(np.stack([g.reshape(-1) for g in grid], 1))).to(dev)
        self.sht = native.Sht(L, device=dev.index)
        if fp64_tables is not None:
            self.sht.set_tables(native.Sht.TABLES_ALWAYS if fp64_tables else native.Sht.TABLES_NEVER)
        if split:
            self.precision_mode = native.Sht.SPLIT_BF16
            src = resources.sht_tables(L) if resources is not None else None
            if src is not None:
                self.sht.share_tables(src)
            else:
                self.sht.set_precision(native.Sht.SPLIT_BF16)
                if resources is not None:
                    resources.set_sht_tables(L, self.sht)
        else:
            self.precision_mode = native.Sht.FP64
            tabled = L <= 512 if fp64_tables is None else bool(fp64_tables)
            if resources is not None and tabled:
                src = resources.sht_tables(("fp64", L))
                if src is not None:
                    self.sht.share_tables(src)
                else:
                    resources.set_sht_tables(("fp64", L), self.sht)
        ns = [i for i in range(1, Nt) if i % n_maps == 0]
        ns.append(Nt)
        self.ns = ns
        self.tspan = np.linspace(0, T, Nt, endpoint=False)
        self.dt = self.tspan[1] - self.tspan[0]
        f64 = dict(dtype=torch.float64, device=dev)
        self.jets = self.id_jets.clone()
        self.coeffs_cur = self.mesh.new_coeffs()
        self.stack = [self.mesh.new_coeffs() for _ in ns]
        self.stack_jets = [torch.empty_like(self.id_jets) for _ in ns]
        self.stack_forms = ([torch.zeros((self.mesh.nt, native.Mesh.FORM_STRIDE), **f64) for _ in ns]
                            if forms else None)
        self.vel_coeffs = [self.vm.new_coeffs() for _ in range(3)]
        self.vel_jets = torch.empty((3, 4, self.vm.nv), **f64)
        self.work = torch.empty(native.lib.cmm_advect_workspace(self.mesh.h), **f64)
        self.X = torch.empty_like(self.sample_pts)
        self.omega = torch.empty((L + 1, 2 * L), **f64)
        self.spline = None
        if self.vort.spline_sh is not None:
            from .workloads import real_to_complex_sh
            alm = torch.from_numpy(real_to_complex_sh(self.vort.spline_sh, L)).to(dev)
            self.spline = self.vm.assemble(self.sht.scalar_jets(self.vm, alm))
        self.cos_grid = self.sample_pts[:, 2].reshape(L + 1, 2 * L)
        self.diag0 = None
        self.Nc = 0
        self.ts0 = float(self.tspan[0])
        self.nvs = 1
        self.stepping = False
        self.identity = True
        self.count = 0
        self.step_index = 0
        self.launches = 0
        self._bve = None        # device-driven stepper, made after the bootstrap
        self.graph = None       # CUDA graph of graph_steps steps (capture())
        self.graph_steps = 1

    # ------------------------------------------------------------ pieces
    def _project(self, X, n, rot=None):
        """omega at X -> velocity slot n (inv_Laplacian + project_stream)."""
        rot = self.rot if rot is None else rot
        self.vm.vorticity(self.vort.kind, self.vort.params, X, rot, sh=self.sh, omega=self.omega,
                          spline=self.spline)
        if self.stepping:
            c = self.vel_coeffs
            self.vel_coeffs = [c[1], c[2], c[0]]
        self.sht.velocity(self.vm, self.omega, jets=self.vel_jets)
        self.vm.assemble(self.vel_jets, out=self.vel_coeffs[n])
        self.launches += 1 + 9 + 1

    def _advect(self, scheme, t, prev):
        self.mesh.advect_project(self.vm, self.vel_coeffs[:self.nvs], self.ts0, scheme, t, self.dt,
                                 self.s_pts, self.tan, prev, jets=self.jets, work=self.work)
        self.mesh.assemble(self.jets, out=self.coeffs_cur)
        self.launches += 3

    def _forms(self, n, current):
        """Form records of the first n stack slots (and None for the
        current map when `current`), or None without forms."""
        if self.stack_forms is None:
            return None
        return self.stack_forms[:n] + ([None] if current else [])

    def _sample(self):
        """submaps(curr_map(sample_pts)) (spherical_simulations.py:268)."""
        cs = self.stack[:self.Nc] + [self.coeffs_cur]
        self.mesh.compose(cs, self.sample_pts, out=self.X, forms=self._forms(self.Nc, True))
        self.launches += 1
        return self.X

    # ------------------------------------------------------------ driver
    def bootstrap(self):
        """spherical_simulations.py:216-261."""
        dt = self.dt
        self._project(self.sample_pts, 0, rot=0.0)   # omega0 on the grid itself
        self.diag0 = self.invariants()
        self._advect(native.EULER, 0.0, None)
        self._project(self._sample_single(), 1)
        self.nvs = 2
        self._advect(native.IMPROVED_EULER, 0.0, None)
        self._project(self._sample_single(), 1)
        prev = self.coeffs_cur.clone()
        self._advect(native.RK4, dt, prev)
        X = self._sample_single()
        self.nvs = 3
        self._project(X, 2)
        self.stepping = True
        self.identity = False
        self.count = 2
        self.step_index = 2
        self._make_stepper()

    def _sample_single(self):
        self.mesh.compose([self.coeffs_cur], self.sample_pts, out=self.X)
        self.launches += 1
        return self.X

    def _make_stepper(self):
        """The device-driven step (cmm_bve_create) from the post-bootstrap state."""
        d = native.BveDesc()
        d.mesh, d.velmesh, d.sht = self.mesh.h, self.vm.h, self.sht.h
        d.vort_kind = self.vort.kind
        d.nparams = len(self.vort.params)
        for k, v in enumerate(self.vort.params[:12]):
            d.vort_params[k] = float(v)
        d.sh = self.sh.data_ptr() if self.sh is not None else None
        d.lmax = self.sh.shape[0] - 1 if self.sh is not None else -1
        d.spline = self.spline.data_ptr() if self.spline is not None else None
        d.rot_rate = float(self.rot)
        d.tspan_step = float(self.dt)
        d.Nt, d.n_maps, d.eps = self.Nt, self.n_maps, 1e-5
        for name in ("s_pts", "tan", "id_jets", "sample_pts", "jets", "coeffs_cur", "work", "X",
                     "omega", "vel_jets"):
            setattr(d, name, getattr(self, name).data_ptr())
        for k in range(3):
            d.vel[k] = self.vel_coeffs[k].data_ptr()
        self._stack_arr = (ctypes.c_void_p * len(self.stack))(*[c.data_ptr() for c in self.stack])
        self._jets_arr = (ctypes.c_void_p * len(self.stack))(*[j.data_ptr() for j in self.stack_jets])
        if self.stack_forms is not None:
            self._forms_arr = (ctypes.c_void_p * len(self.stack))(*[f.data_ptr() for f in self.stack_forms])
            d.stack_forms = ctypes.cast(self._forms_arr, ctypes.c_void_p)
        d.n_stack = len(self.stack)
        d.stack = ctypes.cast(self._stack_arr, ctypes.c_void_p)
        d.stack_jets = ctypes.cast(self._jets_arr, ctypes.c_void_p)
        d.k, d.count, d.nc, d.identity = self.step_index, self.count, self.Nc, int(self.identity)
        d.ts0 = float(self.ts0)
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            native.check(native.lib.cmm_bve_create(ctypes.byref(d), ctypes.byref(h)), "cmm_bve_create")
        self._bve = h

    def __del__(self):
        h = getattr(self, "_bve", None)
        if h is not None and h.value:
            native.lib.cmm_bve_destroy(h)
            self._bve = None

    def _advance_host(self):
        """Host mirror of the driver's bookkeeping (spherical_simulations.py:
        273-294), kept in step with the device state."""
        self.ts0 = self.ts0 + self.dt
        self.count += 1
        self.identity = False
        c = self.vel_coeffs
        self.vel_coeffs = [c[1], c[2], c[0]]
        if self.count in self.ns:
            self.Nc = self.ns.index(self.count) + 1
            self.identity = True
        self.step_index += 1
        self.launches += 13

    def step(self):
        """One pass of the main loop (spherical_simulations.py:263-294),
        enqueued by the device-driven stepper (or replayed from the captured
        CUDA graph after capture())."""
        if self._bve is None:
            self._make_stepper()
        if self.graph is not None:
            self.graph.replay()
            for _ in range(self.graph_steps):
                self._advance_host()
            return
        native.check(native.lib.cmm_bve_step(self._bve, native._stream(self.device)), "cmm_bve_step")
        self._advance_host()

    def capture(self, steps=1):
        """Capture `steps` device-driven steps into one CUDA graph; step()
        then replays it (one graph launch per `steps` steps; the whole
        remaining run when steps = Nt - 2 - count)."""
        if self._bve is None:
            self._make_stepper()
        g = torch.cuda.CUDAGraph()
        torch.cuda.synchronize(self.device)
        with torch.cuda.graph(g):
            for _ in range(steps):
                native.check(native.lib.cmm_bve_step(self._bve, native._stream(self.device)), "cmm_bve_step")
        self.graph, self.graph_steps = g, steps
        return self

    def step_host(self):
        """The same step driven from the host through the single calls
        (advect_project, assemble, compose, vorticity, velocity).  The
        device-driven stepper (and any captured graph) is dropped and made
        again from the host state at the next step()."""
        if self._bve is not None:
            native.lib.cmm_bve_destroy(self._bve)
            self._bve, self.graph = None, None
        t = float(self.tspan[self.step_index])
        self._advect(native.RK4, t, None if self.identity else self.coeffs_cur)
        self._project(self._sample(), 2)
        self.ts0 = self.ts0 + self.dt
        self.count += 1
        self.identity = False
        if self.count in self.ns:
            idx = self.ns.index(self.count)
            self.Nc = idx + 1
            self.stack[idx].copy_(self.coeffs_cur)
            if self.stack_forms is not None:
                self.mesh.assemble_forms(self.stack[idx], out=self.stack_forms[idx])
            self.stack_jets[idx].copy_(self.jets)
            self.jets.copy_(self.id_jets)
            self.identity = True
        self.step_index += 1

    def run(self, nsteps=None):
        self.bootstrap()
        n = self.Nt - 2 if nsteps is None else nsteps
        for _ in range(n):
            self.step()
        return self

    # ----------------------------------------------------- diagnostics
    def invariants(self):
        """Enstrophy and energy of the absolute vorticity omega + 2 Omega
        cos(theta) on the MWSS grid, from its FP64 transform
        (figures/data_gen_convergence.py:58-62, 90-95):
        enstrophy = sum_lm |w_lm|^2, energy = 0.5 (p_0 + sum_l p_l / (l(l+1)))
        with p_l = sum_m |w_lm|^2 (energy_spectrum,
        core/spherical_harmonic_tools.py:157-163)."""
        mode = self.precision_mode
        if mode != native.Sht.FP64:
            self.sht.set_precision(native.Sht.FP64)
        try:
            alm = self.sht.forward(self.omega + 2.0 * self.rot * self.cos_grid)
            p = self.sht.power(alm)
        finally:
            if mode != native.Sht.FP64:
                self.sht.set_precision(mode)
        ell = torch.arange(1, self.L, dtype=torch.float64, device=p.device)
        return {"enstrophy": float(p.sum()),
                "energy": float(0.5 * (p[0] + (p[1:] / (ell * (ell + 1))).sum()))}

    def diagnostics(self, omega_true=None, jacobian=True):
        """Accuracy and conservation of the current state on the MWSS grid:
        enstrophy / energy and their drift relative to t = 0; with
        omega_true (exact relative vorticity on the grid, (L+1, 2L)) the
        L_inf and L2 errors relative to max |omega_true| and its RMS
        (data_gen_convergence.py:84-86); with `jacobian`, the largest
        deviation of the back-to-label map's tangent Jacobian determinant
        from 1 over the sample points (the map is area preserving)."""
        d = self.invariants()
        if self.diag0 is not None:
            d["enstrophy_drift"] = abs(d["enstrophy"] - self.diag0["enstrophy"]) / self.diag0["enstrophy"]
            d["energy_drift"] = abs(d["energy"] - self.diag0["energy"]) / self.diag0["energy"]
        if omega_true is not None:
            ot = torch.as_tensor(omega_true, dtype=torch.float64, device=self.device)
            err = (self.omega - ot).abs()
            d["linf_rel"] = float(err.max() / ot.abs().max())
            d["l2_rel"] = float(err.pow(2).mean().sqrt() / ot.pow(2).mean().sqrt())
        if jacobian:
            x = self.sample_pts
            X, J = self.composite(x, want_jac=True)
            if J is None:
                d["jac_det_dev"] = 0.0
            else:
                a = torch.zeros_like(x)
                a[:, 0] = 1.0
                a[x[:, 0].abs() > 0.9, 0] = 0.0
                a[x[:, 0].abs() > 0.9, 1] = 1.0
                t1 = torch.linalg.cross(a, x)
                t1 = t1 / t1.norm(dim=1, keepdim=True)
                t2 = torch.linalg.cross(x, t1)
                j1 = torch.einsum("nij,nj->ni", J, t1)
                j2 = torch.einsum("nij,nj->ni", J, t2)
                n = X / X.norm(dim=1, keepdim=True)
                det = (n * torch.linalg.cross(j1, j2)).sum(1)
                d["jac_det_dev"] = float((det - 1.0).abs().max())
        return d

    # --------------------------------------------------------- outputs
    def composite(self, q, want_jac=False):
        """The back-to-label map at points q (N,3) on the device: the
        submaps composed with the current map, or the submaps alone right
        after a remap (the reference returns ``submaps``, :297)."""
        cs = self.stack[:self.Nc] + ([] if self.identity else [self.coeffs_cur])
        if not cs:
            return q.clone(), None
        out, _, _, jac = self.mesh.compose(cs, q, want_jac=want_jac,
                                           forms=self._forms(self.Nc, not self.identity))
        return out, jac

    def stack_coeffs(self):
        return self.stack[:self.Nc]

    def submaps(self, mesh):
        """The reference driver's return value (:297): a
        composite_sphere_diffeomorphism over the remapped submaps (jets,
        coefficient records, ns, Nc) on `mesh`, the spherical_triangulation
        this run was built from."""
        from .spherical_spline import composite_sphere_diffeomorphism
        comp = composite_sphere_diffeomorphism(mesh, [j.clone() for j in self.stack_jets],
                                               coeffs=[c.clone() for c in self.stack], ns=list(self.ns))
        comp.Nc = self.Nc
        return comp

    # ------------------------------------------------- checkpoint/resume
    def save_state(self, path):
        """Checkpoint between steps (state_io.save_bve_state)."""
        from .state_io import save_bve_state
        save_bve_state(self, path)

    def load_state(self, path):
        """Resume a checkpoint into this (not bootstrapped) solver."""
        from .state_io import load_bve_state
        return load_bve_state(self, path)


def _solver_for(mesh, L, Nt, T, vorticity, rot_rate, n_maps, precision):
    return BVESolver(mesh.vertices, mesh.simplices, mesh.level, L, Nt, T, vorticity, rot_rate=rot_rate,
                     n_maps=n_maps, device=mesh.device.index, precision=precision)


def euler_simulation_sphere_remapping(L, Nt, T, mesh, vorticity, rot_rate=2 * np.pi, n_maps=10,
                                      precision="fp64"):
    """The reference driver (spherical_simulations.py:144-297) on the GPU:
    `mesh` a spherical_triangulation of this package, `vorticity` a
    reference field function (or its name, or a Vorticity); returns the
    composite_sphere_diffeomorphism of the remapped submaps."""
    s = _solver_for(mesh, L, Nt, T, vorticity, rot_rate, n_maps, precision).run()
    return s.submaps(mesh)


def euler_simulation_sphere(L, Nt, T, mesh, vorticity, rot_rate=2 * np.pi, precision="fp64"):
    """The driver without remapping (spherical_simulations.py:20-141, whose
    own body cannot run: it reads ``mesh_u.verticess``, :56): one map
    over the whole run, returned as a sphere_diffeomorphism."""
    from .spherical_spline import sphere_diffeomorphism
    s = _solver_for(mesh, L, Nt, T, vorticity, rot_rate, Nt, precision).run()
    return sphere_diffeomorphism(mesh, s.stack_jets[0].clone(), s.stack[0].clone())


def euler_simulation_sphere_remapping_video(L, Nt, T, mesh, vorticity, rot_rate, n_maps, file_name, save_steps,
                                            precision="fp64"):
    """spherical_simulations.py:301-457: the remapping driver that also
    writes the current map every `save_steps` steps (except at remaps) as
    the reference's snapshot pickle ``file_name + "<count>.txt"`` =
    {"vals": (3,4,Nv), "Nc"}.  The final submap stack goes to
    ``file_name + "_all_maps.npz"`` (vals, ns, Nc, mesh) instead of a
    pickled reference object.  Returns the composite, as the remapping
    driver."""
    from .state_io import write_reference_snapshot, write_submaps
    s = _solver_for(mesh, L, Nt, T, vorticity, rot_rate, n_maps, precision)
    s.bootstrap()
    for _ in range(Nt - 2):
        s.step()
        if s.count % save_steps == 0 and s.count not in s.ns:
            write_reference_snapshot(file_name + "%s" % s.count + ".txt", s.jets, s.Nc)
    write_submaps(file_name + "_all_maps.npz", s.stack_jets, s.ns, s.Nc, mesh.vertices, mesh.simplices)
    return s.submaps(mesh)
