"""On-disk state of CMM runs.

* Checkpoint / resume of a BVESolver (``save_bve_state`` /
  ``load_bve_state``): one ``.npz`` holding every piece of state the next
  step reads -- the current map's jets, the remapped submaps' jets, the
  three velocity-level records (in the solver's slot order), the counters
  (tspan index, step count, submap count, identity flag), the oldest
  velocity time level, the last vorticity field and the t = 0 invariants --
  plus the configuration it belongs to, checked on load.  A resumed run
  continues bit for bit as if it had not stopped.
* The reference's files: its snapshot dicts ``{"vals": (3,4,Nv), "Nc"}``
  (cmm_s2/core/spherical_simulations.py:434-439) are written and read as
  the reference writes them; its pickled ``composite_sphere_diffeomorphism``
  (:453-455) and pickled meshes are read with a restricted unpickler that
  builds no reference or scipy object (every class the file names is
  replaced by an inert record of its attributes; names outside numpy and
  the reference's own package are refused).
"""
import io
import pickle

import numpy as np
import torch

FORMAT = "cmm-gpu-bve-state/1"


# ------------------------------------------------------ checkpoint/resume
def _config(s):
    return dict(level=int(s.level), L=int(s.L), Nt=int(s.Nt), T=float(s.T), n_maps=int(s.n_maps),
                rot=float(s.rot), precision=int(s.precision_mode), vort_kind=int(s.vort.kind),
                vort_params=np.asarray(s.vort.params, dtype=np.float64), nv=int(s.mesh.nv))


def save_bve_state(solver, path):
    """Write a resumable checkpoint of a bootstrapped solver (between steps)."""
    s = solver
    if not s.stepping:
        raise RuntimeError("save_bve_state: bootstrap the run first")
    torch.cuda.synchronize(s.device)
    cfg = _config(s)
    arrays = {f"cfg_{k}": np.asarray(v) for k, v in cfg.items()}
    arrays.update(
        format=np.asarray(FORMAT), jets=s.jets.cpu().numpy(),
        stack_jets=np.stack([j.cpu().numpy() for j in s.stack_jets[:s.Nc]]) if s.Nc else
        np.zeros((0,) + tuple(s.jets.shape)),
        vel=np.stack([c.cpu().numpy() for c in s.vel_coeffs]),
        omega=s.omega.cpu().numpy(), ts0=np.float64(s.ts0), count=np.int64(s.count),
        step_index=np.int64(s.step_index), Nc=np.int64(s.Nc), identity=np.int64(s.identity),
        nvs=np.int64(s.nvs), diag0=np.asarray([s.diag0[k] for k in sorted(s.diag0)] if s.diag0 else []),
        diag0_keys=np.asarray(sorted(s.diag0) if s.diag0 else []))
    np.savez(path, **arrays)


def load_bve_state(solver, path):
    """Resume a run: `solver` was built with the same configuration and is
    not bootstrapped; after this call step()/run-loop continue the saved run."""
    s = solver
    d = np.load(path, allow_pickle=False)
    if str(d["format"]) != FORMAT:
        raise ValueError(f"{path}: not a {FORMAT} file")
    cfg = _config(s)
    for k, v in cfg.items():
        saved = d[f"cfg_{k}"]
        if not np.array_equal(np.asarray(v), saved):
            raise ValueError(f"{path}: saved {k} = {saved!r}, this solver has {v!r}")
    dev = s.device
    s.jets.copy_(torch.from_numpy(d["jets"]).to(dev))
    s.mesh.assemble(s.jets, out=s.coeffs_cur)
    Nc = int(d["Nc"])
    for i in range(Nc):
        s.stack_jets[i].copy_(torch.from_numpy(d["stack_jets"][i]).to(dev))
        s.mesh.assemble(s.stack_jets[i], out=s.stack[i])
        if s.stack_forms is not None:
            s.mesh.assemble_forms(s.stack[i], out=s.stack_forms[i])
    for k in range(3):
        s.vel_coeffs[k].copy_(torch.from_numpy(d["vel"][k]).to(dev))
    s.omega.copy_(torch.from_numpy(d["omega"]).to(dev))
    s.ts0 = float(d["ts0"])
    s.count, s.step_index, s.Nc = int(d["count"]), int(d["step_index"]), Nc
    s.identity, s.nvs = bool(int(d["identity"])), int(d["nvs"])
    s.diag0 = {str(k): float(v) for k, v in zip(d["diag0_keys"], d["diag0"])} or None
    s.stepping = True
    s._bve, s.graph = None, None
    torch.cuda.synchronize(dev)
    return s


# ------------------------------------------------------ reference files
def write_reference_snapshot(path, vals, Nc):
    """The reference's snapshot file: pickle of {"vals": (3,4,Nv) float64
    ndarray, "Nc": int} (spherical_simulations.py:434-439)."""
    vals = vals.cpu().numpy() if isinstance(vals, torch.Tensor) else np.asarray(vals, dtype=np.float64)
    with open(path, "wb") as f:
        pickle.dump({"vals": np.ascontiguousarray(vals), "Nc": int(Nc)}, f)


class RefRecord:
    """Attributes of an object of a reference class read from a pickle."""

    def __init__(self, *args):
        self._args = args

    def __setstate__(self, state):
        if isinstance(state, tuple) and len(state) == 2 and isinstance(state[1], dict):
            state = {**(state[0] or {}), **state[1]}   # (dict, slots) form
        if isinstance(state, dict):
            self.__dict__.update(state)
        else:
            self._state = state

    def __repr__(self):
        return f"<{type(self).__name__} {sorted(k for k in self.__dict__ if not k.startswith('_'))}>"


_NUMPY = {("numpy.core.multiarray", "_reconstruct"), ("numpy._core.multiarray", "_reconstruct"),
          ("numpy.core.multiarray", "scalar"), ("numpy._core.multiarray", "scalar"),
          ("numpy", "ndarray"), ("numpy", "dtype"), ("numpy.core.numeric", "_frombuffer"),
          ("numpy._core.numeric", "_frombuffer")}
_RECORD_MODULES = ("cmm_s2.", "scipy.spatial")
_BUILTINS = {("builtins", "complex"), ("builtins", "slice"), ("builtins", "range"), ("builtins", "set"),
             ("builtins", "frozenset"), ("copyreg", "_reconstructor"), ("builtins", "object")}


class _RefUnpickler(pickle.Unpickler):
    def find_class(self, module, name):
        if (module, name) in _NUMPY or (module, name) in _BUILTINS:
            return super().find_class(module, name)
        if module.startswith(_RECORD_MODULES):
            return type(name, (RefRecord,), {"__module__": "cmm_gpu.state_io.ref." + module})
        raise pickle.UnpicklingError(f"refusing to load {module}.{name} from a reference file")


def read_reference_pickle(path):
    """Load a pickle written by the reference (snapshot dict, submaps,
    mesh); reference and scipy objects come back as RefRecord instances."""
    with open(path, "rb") as f:
        data = f.read()
    return _RefUnpickler(io.BytesIO(data)).load()


def read_reference_snapshot(path):
    d = read_reference_pickle(path)
    return {"vals": np.asarray(d["vals"], dtype=np.float64), "Nc": int(d["Nc"])}


def reference_submaps(obj):
    """The arrays of a reference composite_sphere_diffeomorphism (or of a
    path to its pickle): vertices, simplices (its Qhull row order), vals
    (n_maps,3,4,Nv), coeffs (n_maps,3,19,Nt), ns, Nc."""
    if isinstance(obj, (str, bytes)) or hasattr(obj, "__fspath__"):
        obj = read_reference_pickle(obj)
    mesh = obj.mesh
    return {"vertices": np.asarray(mesh.vertices, dtype=np.float64),
            "simplices": np.asarray(mesh.simplices, dtype=np.int32),
            "vals": np.asarray(obj.vals, dtype=np.float64), "coeffs": np.asarray(obj.coeffs, dtype=np.float64),
            "ns": [int(n) for n in obj.ns], "Nc": int(obj.Nc)}


def composite_from_reference(obj, device=None):
    """A reference submap stack on the GPU: (spherical_triangulation with the
    reference's triangle table, composite_sphere_diffeomorphism with its
    first Nc submaps assembled)."""
    from .mesh_functions import spherical_triangulation
    from .spherical_spline import composite_sphere_diffeomorphism
    r = reference_submaps(obj)
    mesh = spherical_triangulation(r["vertices"], r["simplices"], device=device)
    comp = composite_sphere_diffeomorphism(mesh, r["vals"], ns=r["ns"])
    for i in range(r["Nc"]):
        comp.assemble_coefficients(i, r["vals"][i])
    comp.Nc = r["Nc"]
    return mesh, comp


def write_submaps(path, vals, ns, Nc, vertices=None, simplices=None):
    """The submap stack in a plain .npz (vals (n,3,4,Nv), ns, Nc, and the
    mesh when given): what the reference's composite_sphere_diffeomorphism
    is built from (spherical_spline.py:355-362)."""
    vals = np.stack([v.cpu().numpy() if isinstance(v, torch.Tensor) else np.asarray(v) for v in vals])
    extra = {}
    if vertices is not None:
        extra["vertices"] = np.asarray(vertices, dtype=np.float64)
    if simplices is not None:
        extra["simplices"] = np.asarray(simplices, dtype=np.int32)
    np.savez(path, vals=vals, ns=np.asarray(ns, dtype=np.int64), Nc=np.int64(Nc), **extra)
