"""Project-written autotuner: launch shapes and compiled variants of the
tunable kernels per size class, the split-BF16 synthesis schedule per
band-limit, and the schedule (branch count, member order) of an
ensemble's captured graph, chosen from CUDA-event timings on the run's own
data.

What is tuned, and what is fixed by the data:
* threads per block of the composition, the map update's foot points and
  the vorticity kernel (cmm_mesh_set_block);
* the composition's register budget (cmm_mesh_set_variant: resident
  blocks 4 or 6 for points only, 2, 3 or 4 with Jacobians) -- the same
  arithmetic compiled for another register count, so results do not
  change -- and, for a query set, whether the queries are grouped by
  coarse cell before the composition (tune_composition);
* the synthesis schedule (cmm_sht_set_schedule: one role per phase, or
  warp-specialised; bitwise the same results), for all plans of a
  band-limit at once (tune_sht_schedule);
* the graph's branch count and member order, and whether the
  same-band-limit members' forward analyses run batched (one tensor-core
  launch per batch of up to 8; bitwise the same results).
The tensor-core tiles are fixed by the data: N = 32 columns holds the
synthesis' 24 real columns (12 complex fields; N = 16 the analysis' 2 per
field, up to 8 fields when batched),
M = 128 the TMEM lanes, and K = 64 the chunk of the Pbar table images the
MMAs read straight from shared memory (another K needs other tables).

Launch shapes (cmm_mesh_set_block) are set per mesh, i.e. per mesh level
(composition, foot points) or band-limit (vorticity); every member of a
size class shares the mesh and so the choice.  Candidates are timed on
scratch outputs (the members' state is not touched).  A schedule candidate
is timed by replaying its graph: those replays are real steps of the run
(results do not depend on the schedule: every kernel is deterministic and
the members are independent), so tuning costs no extra steps.
"""
import json

import torch

from . import native


def _time(fn, reps, stream):
    fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


class Autotuner:
    BLOCKS = (64, 128, 192, 256)
    COMPOSE_VARIANTS = (4, 6)

    def __init__(self, reps=3):
        self.reps = reps
        self.log = {"kernels": {}, "schedule": None}

    # ------------------------------------------------------------ kernels
    def tune_solver(self, s):
        """Launch shapes for the size class (level, L) of solver s, after
        its bootstrap; returns {kernel: (best threads, {threads: ms})}."""
        dev = s.device
        stream = torch.cuda.current_stream(dev)
        X = torch.empty_like(s.X)
        om = torch.empty_like(s.omega)
        jets = torch.empty_like(s.jets)
        work = torch.empty_like(s.work)
        cs = s.stack[:s.Nc] + [s.coeffs_cur]
        t = float(s.tspan[s.step_index])
        prev = None if s.identity else s.coeffs_cur
        stages = {
            native.Mesh.TUNE_COMPOSE: (s.mesh, lambda: s.mesh.compose(cs, s.sample_pts, out=X,
                                                                      forms=s._forms(s.Nc, True))),
            native.Mesh.TUNE_ADVECT: (s.mesh, lambda: s.mesh.advect_project(
                s.vm, s.vel_coeffs, s.ts0, native.RK4, t, s.dt, s.s_pts, s.tan, prev, jets=jets,
                work=work)),
            native.Mesh.TUNE_VORTICITY: (s.vm, lambda: s.vm.vorticity(
                s.vort.kind, s.vort.params, s.X, s.rot, sh=s.sh, omega=om, spline=s.spline)),
        }
        out = {}
        for k, (mesh, fn) in stages.items():
            times = {}
            for b in self.BLOCKS:
                mesh.set_block(k, b)
                times[b] = _time(fn, self.reps, stream)
            best = min(times, key=times.get)
            mesh.set_block(k, best)
            out[k] = (best, times)
        # register budget of the grid composition (same results)
        compose = stages[native.Mesh.TUNE_COMPOSE][1]
        vt = {}
        for v in self.COMPOSE_VARIANTS:
            s.mesh.set_variant(native.Mesh.VARIANT_COMPOSE, v)
            vt[v] = _time(compose, self.reps, stream)
        vbest = min(vt, key=vt.get)
        s.mesh.set_variant(native.Mesh.VARIANT_COMPOSE, vbest)
        self.log.setdefault("variants", {})[f"level{s.level}_L{s.L}"] = {"compose_blocks": vbest, "ms": vt}
        self.log["kernels"][f"level{s.level}_L{s.L}"] = {
            name: {"best": out[k][0], "ms": out[k][1]}
            for name, k in (("compose", 0), ("advect", 1), ("vorticity", 2))}
        return out

    def tune_ensemble_kernels(self, ens):
        """One representative member (the first) per (level, L) class."""
        seen = set()
        for m in ens.members:
            key = (m.level, m.L)
            if key in seen:
                continue
            seen.add(key)
            self.tune_solver(m)
        return self.log["kernels"]

    # ------------------------------------------------------ composition
    def tune_composition(self, mesh, step, stream, variants=(2, 3, 4), orders=(True, False), reps=3):
        """Register budget of the Jacobian composition (cmm_mesh_set_variant,
        resident blocks per SM: the same arithmetic compiled for another
        register count, so results do not change) and whether the queries
        are grouped by coarse cell first, from CUDA-event timings of
        `step(ordered)` (one composition step on the caller's data, the
        sort included when ordered).  Sets the best variant on the mesh and
        returns the best order; the timings go to log["composition"]."""
        times = {}
        for v in variants:
            mesh.set_variant(native.Mesh.VARIANT_COMPOSE_JAC, v)
            for o in orders:
                times[(v, o)] = _time(lambda: step(o), reps, stream)
        (vb, ob) = min(times, key=times.get)
        mesh.set_variant(native.Mesh.VARIANT_COMPOSE_JAC, vb)
        self.log["composition"] = {"compose_jac_blocks": vb, "ordered": ob,
                                   "ms": {f"blocks{v}_{'cell' if o else 'caller'}": t
                                          for (v, o), t in times.items()}}
        return ob

    # ------------------------------------------------- synthesis schedule
    def tune_sht_schedule(self, solvers, reps=3):
        """Split-BF16 synthesis schedule per band-limit, timed on the first
        solver of each L (its own velocity step) and applied to every
        solver of that L."""
        byL = {}
        for s in solvers:
            if s.precision_mode == native.Sht.SPLIT_BF16:
                byL.setdefault(s.L, []).append(s)
        res = {}
        for L, group in byL.items():
            s = group[0]
            stream = torch.cuda.current_stream(s.device)
            jets = torch.empty_like(s.vel_jets)
            times = {}
            for sched in (native.Sht.SCHEDULE_PER_CHUNK, native.Sht.SCHEDULE_WARP_SPECIALISED):
                s.sht.set_schedule(sched)
                times[sched] = _time(lambda: s.sht.velocity(s.vm, s.omega, jets=jets), reps, stream)
            best = min(times, key=times.get)
            for m in group:
                m.sht.set_schedule(best)
            res[f"L{L}"] = {"schedule": best, "ms": times}
        self.log["sht_schedule"] = res
        return res

    # ----------------------------------------------------------- schedule
    def tune_schedule(self, ens, stream_counts=(1, 2, 4, 8), steps_each=2, batch=True):
        """Capture the ensemble's graph for each branch count and member
        order (as given; largest work first) and time `steps_each` replays
        of each; then (batch) the best of them with the same-band-limit
        members' analyses batched (Ensemble.capture(batch=True)); keep the
        fastest.  Returns the timings."""
        work = [m.sample_pts.shape[0] * (1 + m.n_maps) + m.mesh.nv * 20 for m in ens.members]
        orders = {"given": list(range(len(ens.members))),
                  "largest_first": sorted(range(len(ens.members)), key=lambda i: -work[i])}
        stream = torch.cuda.current_stream(ens.device)
        results = []
        for name, order in orders.items():
            for ns in stream_counts:
                ens.capture(streams=ns, order=order)
                torch.cuda.synchronize()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                for _ in range(steps_each):
                    ens.step()
                e1.record(stream)
                torch.cuda.synchronize()
                results.append({"order": name, "streams": ns, "ms_per_step": e0.elapsed_time(e1) / steps_each})
        best = min(results, key=lambda r: r["ms_per_step"])
        for r in results:
            r["batch"] = False
        # the same-band-limit members' analyses batched (one tensor-core
        # launch per batch), on the best unbatched schedule
        if batch and ens.batches()[1]:
            ens.capture(streams=best["streams"], order=orders[best["order"]], batch=True)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(steps_each):
                ens.step()
            e1.record(stream)
            torch.cuda.synchronize()
            rb = {"order": best["order"], "streams": best["streams"], "batch": True,
                  "ms_per_step": e0.elapsed_time(e1) / steps_each}
            results.append(rb)
            if rb["ms_per_step"] < best["ms_per_step"]:
                best = rb
        ens.capture(streams=best["streams"], order=orders[best["order"]], batch=best["batch"])
        self.log["schedule"] = {"best": best, "candidates": results}
        return self.log["schedule"]

    def save(self, path):
        with open(path, "w") as f:
            json.dump(self.log, f, indent=1)
