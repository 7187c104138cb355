"""Ensembles of barotropic runs of uneven sizes advanced together on one GPU.

Each member is a BVESolver (its own map stack, velocity levels, vorticity
and transform scratch); members of the same mesh level share the map mesh
and its stencil frames, members of the same band-limit share the velocity
mesh and the split-BF16 Pbar tables.  After every member's bootstrap, one
device-driven step of all members (cmm_bve_step, whose varying state lives
on the device) is captured into ONE CUDA graph, the members spread over
parallel branches; every later step of the whole ensemble is one replay of
that graph, or the whole remaining run is captured as one graph and
launched once (run_persistent).  The branch count and member order of the graph and the launch
shapes of the tunable kernels of each size class are chosen by the
Autotuner from measured timings.

No counterpart in the reference, which runs one simulation per process
(cmm_s2/core/spherical_simulations.py); each member reproduces that
driver's run.
"""
import time

import numpy as np
import torch

from . import native
from .meshgen import icosahedral_mesh, latlon_mesh_arrays, stencil_frames, identity_jets
from .spherical_simulations import BVESolver, Vorticity
from .workloads import spectral_perturbation


class SharedResources:
    """Read-only objects shared by the members: map meshes and stencil
    frames per level, velocity meshes per band-limit (and record
    precision), the MWSS sample points and the Legendre table owners
    (split-BF16 and FP64) per band-limit."""

    def __init__(self, device):
        self.device = device
        self._mesh, self._frames, self._vm, self._grid, self._sht = {}, {}, {}, {}, {}

    def mesh(self, level):
        if level not in self._mesh:
            verts, tris = icosahedral_mesh(level)
            self._mesh[level] = (verts, tris, native.Mesh(verts, tris, level, device=self.device.index))
        return self._mesh[level]

    def frames(self, level):
        if level not in self._frames:
            verts = self.mesh(level)[0]
            tan, s_pts = stencil_frames(verts)
            dev = self.device
            self._frames[level] = (torch.from_numpy(np.ascontiguousarray(tan)).to(dev),
                                   torch.from_numpy(np.ascontiguousarray(s_pts)).to(dev),
                                   torch.from_numpy(identity_jets(verts)).to(dev))
        return self._frames[level]

    def velmesh(self, L, rec32):
        key = (L, rec32)
        if key not in self._vm:
            theta, phi, grid, vverts = latlon_mesh_arrays(L)
            vm = native.VelMesh(L, theta, phi, grid, vverts, device=self.device.index)
            if rec32:
                vm.set_records(native.VelMesh.REC_MIXED)
            self._vm[key] = (vm, grid)
        return self._vm[key]

    def sample_pts(self, L):
        if L not in self._grid:
            grid = latlon_mesh_arrays(L)[2]
            self._grid[L] = torch.from_numpy(
                np.ascontiguousarray(np.stack([g.reshape(-1) for g in grid], 1))).to(self.device)
        return self._grid[L]

    def sht_tables(self, L):
        """The plan holding the split-BF16 tables of band-limit L (key L), or
        the FP64 Pbar tables (key ("fp64", L)), or None."""
        return self._sht.get(L)

    def set_sht_tables(self, L, sht):
        self._sht.setdefault(L, sht)


# Map forms pay when the evaluations through a remapped submap outnumber
# the triangles by more than this factor: assembling a submap's forms costs
# 6.1 ms per 327,680 triangles (18.6 ns per triangle, double-double on the
# FP64 pipe), and each evaluation through a form instead of a coefficient
# record saves ~20 FP64 instructions (26.8 against 46.5), 32 ps at the
# measured 0.63 x 10^12 FP64 instructions/s.
FORMS_EVALS_PER_TRIANGLE = 582


def forms_pay(level, L, Nt, n_maps):
    """Whether map forms pay for a run of Nt steps at mesh level `level` and
    band-limit L remapping every n_maps steps: the (L+1) x 2L sample points
    pass through each remapped submap on every later step (on average the
    remaining half of the run)."""
    points = (L + 1) * 2 * L
    remaps = [i for i in range(1, Nt) if i % n_maps == 0]
    if not remaps:
        return False
    later = sum(Nt - i for i in remaps) / len(remaps)
    return points * later > FORMS_EVALS_PER_TRIANGLE * (20 << (2 * level))


class Ensemble:
    def __init__(self, members):
        self.members = list(members)
        self.device = self.members[0].device
        self.graph = None
        self.schedule = None
        self.count = 0
        self._batch_groups = None

    @classmethod
    def from_seed(cls, n, seed, levels=(5, 6, 7), bandlimits=(256, 512, 1024), Nt=100, T=0.5,
                  lmax=64, rms=5.0, n_maps=10, precision="split_bf16", device=None, forms=None):
        """n members with mesh level and band-limit drawn from `seed`; each
        starts from seeded random vorticity over l <= lmax with a k^-3
        spectrum (coefficients N(0,1) l^-2, scaled to the given RMS),
        evaluated through its scalar spline.  forms: the members' remapped
        submaps with map-form records (BVESolver), True / False for all, or
        None: per member, when they pay (forms_pay) and the chosen members'
        records (0.9 KB per triangle and slot) take at most a quarter of the
        free device memory."""
        device = torch.device("cuda", torch.cuda.current_device() if device is None else device)
        rng = np.random.default_rng(seed)
        specs = [(int(rng.choice(levels)), int(rng.choice(bandlimits))) for _ in range(n)]
        if forms is None:
            use = [forms_pay(lv, L, Nt, n_maps) for lv, L in specs]
            slots = len([i for i in range(1, Nt) if i % n_maps == 0]) + 1
            need = sum(slots * (20 << (2 * lv)) * native.Mesh.FORM_STRIDE * 8
                       for (lv, _), u in zip(specs, use) if u)
            if need > 0.25 * torch.cuda.mem_get_info(device)[0]:
                use = [False] * n
        else:
            use = [bool(forms)] * n
        res = SharedResources(device)
        members = []
        for i, (level, L) in enumerate(specs):
            pert = spectral_perturbation(lmax, seed=seed * 100003 + i, slope=-2.0, rms=rms)
            members.append(BVESolver(None, None, level, L, Nt, T, Vorticity(spline_sh=pert),
                                     n_maps=n_maps, precision=precision, resources=res, forms=use[i]))
        ens = cls(members)
        ens.specs = specs
        ens.resources = res
        return ens

    # ----------------------------------------------------------------
    def bootstrap(self):
        for m in self.members:
            m.bootstrap()
            if m.precision_mode == native.Sht.SPLIT_BF16:
                m.sht.trim()   # FP64 inverse scratch is needed only for the set-up
        torch.cuda.synchronize(self.device)
        return self

    def batches(self):
        """The split-BF16 members grouped by band-limit into batches of up
        to 8 whose forward analyses run as one tensor-core launch
        (native.ShtBatch; a band-limit with one such member stays alone):
        ({member index: batch}, [batches]), made once."""
        if self._batch_groups is None:
            byL = {}
            for i, m in enumerate(self.members):
                if m.precision_mode == native.Sht.SPLIT_BF16:
                    byL.setdefault(m.L, []).append(i)
            of, groups = {}, []
            for L in sorted(byL):
                idx = byL[L]
                for k in range(0, len(idx), native.ShtBatch.MAX):
                    grp = idx[k:k + native.ShtBatch.MAX]
                    if len(grp) < 2:
                        continue
                    b = native.ShtBatch([self.members[i].sht for i in grp])
                    groups.append(b)
                    for i in grp:
                        of[i] = b
            self._batch_groups = (of, groups)
        return self._batch_groups

    def capture(self, streams=4, order=None, steps=1, batch=False):
        """`steps` steps of every member into one CUDA graph: members
        assigned round-robin (in `order`, default as given) to `streams`
        parallel branches forked from and joined into the capture stream;
        each branch runs its members' steps in order (a member's step k+1
        after its step k on the same branch; members never wait on each
        other).  Every step's state lives on the device (cmm_bve_step), so
        the whole remaining run can be one graph: one launch.
        batch: the members of each analysis batch (batches()) run each step
        in two halves (cmm_bve_step_pre / _post) around one batched
        analysis per batch; the branches join before the analyses and
        again before the second halves.  Same results bitwise."""
        order = list(range(len(self.members))) if order is None else list(order)
        of, groups = self.batches() if batch else ({}, [])
        g = torch.cuda.CUDAGraph()
        side = [torch.cuda.Stream(self.device) for _ in range(streams)]
        torch.cuda.synchronize(self.device)

        def join_fork(cap):
            for st in side:
                cap.wait_stream(st)
            for st in side:
                st.wait_stream(cap)

        with torch.cuda.graph(g):
            cap = torch.cuda.current_stream(self.device)
            for st in side:
                st.wait_stream(cap)
            for _ in range(steps):
                for k, i in enumerate(order):
                    with torch.cuda.stream(side[k % streams]):
                        fn, name = ((native.lib.cmm_bve_step_pre, "cmm_bve_step_pre") if i in of else
                                    (native.lib.cmm_bve_step, "cmm_bve_step"))
                        native.check(fn(self.members[i]._bve, native._stream(self.device)), name)
                if groups:
                    join_fork(cap)
                    for j, b in enumerate(groups):
                        with torch.cuda.stream(side[j % streams]):
                            b.analysis(native._stream(self.device))
                    join_fork(cap)
                    for k, i in enumerate(order):
                        if i in of:
                            with torch.cuda.stream(side[k % streams]):
                                native.check(native.lib.cmm_bve_step_post(self.members[i]._bve,
                                                                          native._stream(self.device)),
                                             "cmm_bve_step_post")
            for st in side:
                cap.wait_stream(st)
        self.graph = g
        self.schedule = {"streams": streams, "order": order, "steps": steps, "batch": bool(groups)}
        return self

    def step(self):
        """One graph launch: schedule["steps"] steps of every member."""
        self.graph.replay()
        for _ in range(self.schedule.get("steps", 1)):
            for m in self.members:
                m._advance_host()
            self.count += 1

    def run_persistent(self, nsteps=None):
        """The remaining run (or `nsteps` steps) as one captured graph on the
        current schedule, launched once."""
        n = self.members[0].Nt - 2 - self.count if nsteps is None else nsteps
        sched = self.schedule or {"streams": 4, "order": None}
        self.capture(streams=sched["streams"], order=sched["order"], steps=n, batch=sched.get("batch", False))
        self.step()
        return self

    def run(self, nsteps=None):
        n = self.members[0].Nt - 2 if nsteps is None else nsteps
        per = self.schedule.get("steps", 1) if self.schedule else 1
        if n % per:
            raise ValueError(f"{n} steps is not a multiple of the graph's {per}")
        for _ in range(n // per):
            self.step()
        return self

    def member_steps(self):
        return sum(m.count for m in self.members)

    def memory_bytes(self):
        return torch.cuda.memory_allocated(self.device)
