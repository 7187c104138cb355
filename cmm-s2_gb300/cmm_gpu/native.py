"""ctypes binding of libcmmgpu.so (the C ABI declared in include/cmm_gpu.h).

The library is built in-tree by ``__graft_entry__.build()`` into
``cmm-s2_gb300/lib/libcmmgpu.so``.  There is no fallback: importing this
module without the library, or calling it without a CUDA device, raises.
"""
import ctypes
import os

import numpy as np
import torch

_LIB_PATH = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "lib",
                         "libcmmgpu.so")

if not os.path.exists(_LIB_PATH):
    raise ImportError(f"libcmmgpu.so not built ({_LIB_PATH}); run __graft_entry__.build()")

lib = ctypes.CDLL(_LIB_PATH)

_p, _i, _i64, _d = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_double


class BveDesc(ctypes.Structure):
    """cmm_bve_desc (include/cmm_gpu.h)."""
    _fields_ = [("mesh", _p), ("velmesh", _p), ("sht", _p),
                ("vort_kind", _i), ("nparams", _i), ("vort_params", _d * 12),
                ("sh", _p), ("lmax", _i), ("spline", _p), ("rot_rate", _d),
                ("tspan_step", _d), ("Nt", _i), ("n_maps", _i), ("eps", _d),
                ("s_pts", _p), ("tan", _p), ("id_jets", _p), ("sample_pts", _p),
                ("jets", _p), ("coeffs_cur", _p), ("work", _p), ("X", _p), ("omega", _p),
                ("vel_jets", _p), ("vel", _p * 3), ("n_stack", _i), ("stack", _p),
                ("stack_jets", _p), ("k", _i), ("count", _i), ("nc", _i), ("identity", _i),
                ("ts0", _d), ("stack_forms", _p)]


_SIGS = {
    "cmm_last_error": (ctypes.c_char_p, []),
    "cmm_version": (_i, []),
    "cmm_launch_count": (ctypes.c_longlong, []),
    "cmm_mesh_create": (_i, [_p, _i, _p, _i, _i, ctypes.POINTER(_p)]),
    "cmm_mesh_destroy": (_i, [_p]),
    "cmm_mesh_check": (_i, [_p, _i, _p, _i, _i, _p]),
    "cmm_mesh_status": (_i, [_p, _p, ctypes.POINTER(_i), _i]),
    "cmm_coeff_stride": (_i, [_i]),
    "cmm_locate": (_i, [_p, _p, _i64, _p, _p, _p]),
    "cmm_assemble": (_i, [_p, _p, _i, _p, _p]),
    "cmm_compose": (_i, [_p, ctypes.POINTER(_p), _i, _p, _i64, _p, _p, _p, _p, _p]),
    "cmm_flow_velocity": (_i, [_p, _i, _d, _d, _d, _p, _i64, _p, _p]),
    "cmm_flow_integrate": (_i, [_p, _i, _d, _d, _i, _d, _d, _p, _i64, _p, _p]),
    "cmm_flow_advect_project": (_i, [_p, _i, _d, _d, _i, _d, _d, _p, _p, _p, _d, _p, _p, _p]),
    "cmm_tracer_eval": (_i, [_p, _i, _d, _p, _i64, _p, _p]),
    "cmm_query_order_workspace": (_i64, [_i64]),
    "cmm_query_order": (_i, [_p, _p, _i64, _p, _p, _p]),
    "cmm_compose_ordered": (_i, [_p, ctypes.POINTER(_p), _i, _p, _i64, _p, _p, _p, _p, _p, _p]),
    "cmm_assemble_forms": (_i, [_p, _p, _p, _p]),
    "cmm_forms_ff": (_i, [_p, _p, _p, _p]),
    "cmm_compose_forms": (_i, [_p, ctypes.POINTER(_p), ctypes.POINTER(_p), ctypes.POINTER(_p), _i, _p, _i64,
                               _p, _p, _p, _p, _p, _p]),
    "cmm_stencil_eval": (_i, [_p, _p, _p, _p, _i64, _p, _p]),
    "cmm_velmesh_create": (_i, [_i, _p, _p, _p, _p, ctypes.POINTER(_p)]),
    "cmm_velocity_eval": (_i, [_p, ctypes.POINTER(_p), _i, _d, _d, _d, _p, _i64, _p, _p]),
    "cmm_integrate": (_i, [_p, ctypes.POINTER(_p), _i, _d, _i, _d, _d, _p, _i64, _p, _p]),
    "cmm_advect_workspace": (_i64, [_p]),
    "cmm_vorticity_eval": (_i, [_p, _i, _p, _i, _p, _i, _p, _d, _p, _p, _p]),
    "cmm_sht_scalar_jets": (_i, [_p, _p, _p, _p, _p]),
    "cmm_sht_create": (_i, [_i, ctypes.POINTER(_p)]),
    "cmm_sht_set_precision": (_i, [_p, _i]),
    "cmm_sht_set_schedule": (_i, [_p, _i]),
    "cmm_sht_status": (_i, [_p, _p, ctypes.POINTER(_i), _i]),
    "cmm_sht_power": (_i, [_p, _p, _p, _p]),
    "cmm_sht_share_tables": (_i, [_p, _p]),
    "cmm_sht_trim": (_i, [_p]),
    "cmm_sht_batch_create": (_i, [ctypes.POINTER(_p), _i, ctypes.POINTER(_p)]),
    "cmm_sht_batch_destroy": (_i, [_p]),
    "cmm_sht_batch_analysis": (_i, [_p, _p]),
    "cmm_sht_batch_forward": (_i, [_p, ctypes.POINTER(_p), ctypes.POINTER(_p), _p]),
    "cmm_sht_set_tables": (_i, [_p, _i]),
    "cmm_sht_timeout_selftest": (_i, [_p, _i64, _p]),
    "cmm_velmesh_set_records": (_i, [_p, _i]),
    "cmm_assemble_bwd": (_i, [_p, _p, _p, _p]),
    "cmm_compose_bwd": (_i, [_p, ctypes.POINTER(_p), _i, _p, _i64, _p, ctypes.POINTER(_p), _p, _p, _p]),
    "cmm_vorticity_bwd": (_i, [_p, _p, _i, _d, _p, _p, _p, _p, _p]),
    "cmm_sht_velocity_bwd": (_i, [_p, _p, _p, _p, _p]),
    "cmm_advect_project_bwd": (_i, [_p, _p, ctypes.POINTER(_p), _i, _d, _i, _d, _d, _p, _p, _p, _d, _p,
                                    ctypes.POINTER(_p), _p, _p, _p]),
    "cmm_mesh_set_block": (_i, [_p, _i, _i]),
    "cmm_mesh_set_variant": (_i, [_p, _i, _i]),
    "cmm_bve_create": (_i, [ctypes.POINTER(BveDesc), ctypes.POINTER(_p)]),
    "cmm_bve_destroy": (_i, [_p]),
    "cmm_bve_step": (_i, [_p, _p]),
    "cmm_bve_step_pre": (_i, [_p, _p]),
    "cmm_bve_step_post": (_i, [_p, _p]),
    "cmm_bve_state": (_i, [_p, _p, ctypes.POINTER(_i), ctypes.POINTER(_i), ctypes.POINTER(_i)]),
    "cmm_sht_destroy": (_i, [_p]),
    "cmm_sht_forward": (_i, [_p, _p, _p, _p]),
    "cmm_sht_inverse": (_i, [_p, _p, _i, _p, _p]),
    "cmm_sht_velocity": (_i, [_p, _p, _p, _p, _p, _p]),
    "cmm_advect_project": (_i, [_p, _p, ctypes.POINTER(_p), _i, _d, _i, _d, _d, _p, _p, _p, _d, _p,
                                _p, _p]),
    "cmm_advect_project_noalloc": (_i, [_p, _p, ctypes.POINTER(_p), _i, _d, _i, _d, _d, _p, _p, _p,
                                        _d, _p, _p]),
}
for _name, (_res, _args) in _SIGS.items():
    _f = getattr(lib, _name)
    _f.restype, _f.argtypes = _res, _args

STATUS = {0: "OK", 1: "ERR_ARG", 2: "ERR_MESH", 3: "ERR_CUDA", 4: "ERR_NONFINITE", 5: "ERR_LOCATE",
          6: "ERR_TIMEOUT", 7: "ERR_UNSUPPORTED"}
FLAG_NONFINITE, FLAG_LOCATE, FLAG_TIMEOUT, FLAG_INDEX = 1, 2, 4, 8


class CmmError(RuntimeError):
    def __init__(self, code, where):
        msg = lib.cmm_last_error().decode(errors="replace")
        super().__init__(f"{where}: {STATUS.get(code, code)}: {msg}")
        self.code = code


def check(code, where):
    if code != 0:
        raise CmmError(code, where)


def exported_symbols():
    return sorted(_SIGS)


def mesh_check(verts, tris, level):
    """Host-only hierarchy build; returns the leaf -> row table (no GPU needed)."""
    verts = np.ascontiguousarray(verts, dtype=np.float64)
    tris = np.ascontiguousarray(tris, dtype=np.int32)
    rows = np.empty(len(tris), dtype=np.int32)
    check(lib.cmm_mesh_check(verts.ctypes.data, len(verts), tris.ctypes.data, len(tris), level,
                             rows.ctypes.data), "cmm_mesh_check")
    return rows


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _stream(device=None):
    return ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)


def _dev(t, dtype=torch.float64):
    if not (isinstance(t, torch.Tensor) and t.is_cuda):
        raise TypeError("expected a CUDA tensor")
    if t.dtype != dtype:
        raise TypeError(f"expected {dtype}, got {t.dtype}")
    return t.contiguous()


class Mesh:
    """Device context of an icosahedral mesh (cmm_mesh_create)."""

    def __init__(self, verts, tris, level, device=None):
        verts = np.ascontiguousarray(verts, dtype=np.float64)
        tris = np.ascontiguousarray(tris, dtype=np.int32)
        self.device = torch.device("cuda", torch.cuda.current_device() if device is None else device)
        self.nv, self.nt, self.level = len(verts), len(tris), level
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            check(lib.cmm_mesh_create(verts.ctypes.data, len(verts), tris.ctypes.data, len(tris),
                                      level, ctypes.byref(h)), "cmm_mesh_create")
        self.h = h
        self.stride = lib.cmm_coeff_stride(3)

    def __del__(self):
        h = getattr(self, "h", None)
        if h is not None and h.value:
            lib.cmm_mesh_destroy(h)
            self.h = None

    TUNE_COMPOSE, TUNE_ADVECT, TUNE_VORTICITY, TUNE_LOCATE = 0, 1, 2, 3

    def set_block(self, kernel, threads):
        """Launch shape of a tunable kernel on this mesh (cmm_mesh_set_block)."""
        check(lib.cmm_mesh_set_block(self.h, kernel, threads), "cmm_mesh_set_block")
        return self

    VARIANT_COMPOSE_JAC, VARIANT_COMPOSE = 0, 1

    def set_variant(self, knob, value):
        """Compiled variant (register budget) of a tunable kernel on this
        mesh (cmm_mesh_set_variant)."""
        check(lib.cmm_mesh_set_variant(self.h, knob, value), "cmm_mesh_set_variant")
        return self

    # ------------------------------------------------------------------
    def status(self, clear=True):
        f = ctypes.c_int()
        check(lib.cmm_mesh_status(self.h, _stream(self.device), ctypes.byref(f), int(clear)),
              "cmm_mesh_status")
        return f.value

    def new_coeffs(self, ncomp=3, batch=()):
        return torch.zeros((*batch, self.nt, lib.cmm_coeff_stride(ncomp)), dtype=torch.float64,
                           device=self.device)

    def locate(self, q, want_bcc=True):
        q = _dev(q)
        n = q.shape[0]
        tri = torch.empty(n, dtype=torch.int32, device=q.device)
        bcc = torch.empty((n, 3), dtype=torch.float64, device=q.device) if want_bcc else None
        check(lib.cmm_locate(self.h, _ptr(q), n, _ptr(tri), _ptr(bcc), _stream(q.device)), "cmm_locate")
        return tri, bcc

    def assemble(self, jets, out=None):
        jets = _dev(jets)
        ncomp = jets.shape[0] if jets.dim() == 3 else 1
        if out is None:
            out = self.new_coeffs(ncomp)
        want = torch.float32 if (ncomp == 3 and getattr(self, "rec32", False)) else torch.float64
        if out.dtype != want or not out.is_contiguous():
            raise TypeError(f"cmm_assemble: coefficient records must be contiguous {want}")
        check(lib.cmm_assemble(self.h, _ptr(jets), ncomp, _ptr(out), _stream(jets.device)),
              "cmm_assemble")
        return out

    FORM_STRIDE = 112

    def assemble_forms(self, coeffs, out=None):
        """Map-form records (Nt, 112) of coefficient records (cmm_assemble_forms)."""
        if out is None:
            out = torch.empty((self.nt, self.FORM_STRIDE), dtype=torch.float64, device=coeffs.device)
        check(lib.cmm_assemble_forms(self.h, _ptr(coeffs), _ptr(out), _stream(coeffs.device)),
              "cmm_assemble_forms")
        return out

    FORM_FF_STRIDE = 112

    def forms_ff(self, forms, out=None):
        """Low floats (Nt, 112) float32 of the float-float split of map-form
        records (cmm_forms_ff), read by the Jacobian compositions."""
        if out is None:
            out = torch.empty((self.nt, self.FORM_FF_STRIDE), dtype=torch.float32, device=forms.device)
        check(lib.cmm_forms_ff(self.h, _ptr(forms), _ptr(out), _stream(forms.device)), "cmm_forms_ff")
        return out

    def query_order(self, q, work=None):
        """Permutation grouping the queries by coarse hierarchy cell."""
        q = _dev(q)
        n = q.shape[0]
        perm = torch.empty(n, dtype=torch.int32, device=q.device)
        need = lib.cmm_query_order_workspace(n)
        if work is None or work.numel() < need:
            work = torch.empty(need, dtype=torch.int32, device=q.device)
        check(lib.cmm_query_order(self.h, _ptr(q), n, _ptr(perm), _ptr(work), _stream(q.device)),
              "cmm_query_order")
        return perm

    def compose(self, coeffs, q, want_tri=False, want_tri_all=False, want_jac=False, out=None,
                perm=None, forms=None, forms_ff=None):
        """coeffs: list of coefficient tensors, submap 0 first (applied last).
        perm: optional processing order (query_order), same results.
        forms: optional list of map-form records (entries may be None);
        forms_ff: optional list of their float-float copies (forms_ff())."""
        q = _dev(q)
        n = q.shape[0]
        S = len(coeffs)
        arr = (ctypes.c_void_p * S)(*[c.data_ptr() for c in coeffs])
        out = torch.empty((n, 3), dtype=torch.float64, device=q.device) if out is None else out
        tri = torch.empty(n, dtype=torch.int32, device=q.device) if want_tri else None
        tri_all = torch.empty((S, n), dtype=torch.int32, device=q.device) if want_tri_all else None
        jac = torch.empty((n, 3, 3), dtype=torch.float64, device=q.device) if want_jac else None
        if forms is not None:
            farr = (ctypes.c_void_p * S)(*[None if f is None else f.data_ptr() for f in forms])
            garr = None if forms_ff is None else \
                (ctypes.c_void_p * S)(*[None if g is None else g.data_ptr() for g in forms_ff])
            check(lib.cmm_compose_forms(self.h, arr, farr, garr, S, _ptr(q), n, _ptr(perm), _ptr(out),
                                        _ptr(tri), _ptr(tri_all), _ptr(jac), _stream(q.device)),
                  "cmm_compose_forms")
        elif perm is None:
            check(lib.cmm_compose(self.h, arr, S, _ptr(q), n, _ptr(out), _ptr(tri), _ptr(tri_all),
                                  _ptr(jac), _stream(q.device)), "cmm_compose")
        else:
            check(lib.cmm_compose_ordered(self.h, arr, S, _ptr(q), n, _ptr(perm), _ptr(out), _ptr(tri),
                                          _ptr(tri_all), _ptr(jac), _stream(q.device)),
                  "cmm_compose_ordered")
        return out, tri, tri_all, jac

    def stencil_eval(self, coeffs, yn, st):
        yn, st = _dev(yn), _dev(st)
        nv = yn.shape[1]
        out = torch.empty_like(st)
        check(lib.cmm_stencil_eval(self.h, _ptr(coeffs), _ptr(yn), _ptr(st), nv, _ptr(out),
                                   _stream(yn.device)), "cmm_stencil_eval")
        return out

    def advect_project(self, velmesh, vel_coeffs, ts0, scheme, t, dt, s_pts, tan, prev_coeffs,
                       eps=1e-5, jets=None, work=None):
        """One CMM map update; returns (jets (3,4,nv), work)."""
        s_pts, tan = _dev(s_pts), _dev(tan)
        if jets is None:
            jets = torch.empty((3, 4, self.nv), dtype=torch.float64, device=s_pts.device)
        if work is None:
            work = torch.empty(lib.cmm_advect_workspace(self.h), dtype=torch.float64,
                               device=s_pts.device)
        arr = (ctypes.c_void_p * len(vel_coeffs))(*[c.data_ptr() for c in vel_coeffs])
        check(lib.cmm_advect_project(self.h, velmesh.h, arr, len(vel_coeffs), ts0, scheme, t, dt,
                                     _ptr(s_pts), _ptr(tan), _ptr(prev_coeffs), eps, _ptr(jets),
                                     _ptr(work), _stream(s_pts.device)), "cmm_advect_project")
        return jets, work

    # ---------------------------------------------------- linear transport
    def flow_velocity(self, flow, t, x, T=1.0, alpha=0.0):
        """Analytic flow velocity at x (3,n) -> (3,n)."""
        x = _dev(x)
        out = torch.empty_like(x)
        check(lib.cmm_flow_velocity(self.h, flow, T, alpha, t, _ptr(x), x.shape[1], _ptr(out),
                                    _stream(x.device)), "cmm_flow_velocity")
        return out

    def flow_integrate(self, flow, scheme, t, dt, x, T=1.0, alpha=0.0):
        """Backward foot points of x (3,n) under an analytic flow."""
        x = _dev(x)
        out = torch.empty_like(x)
        check(lib.cmm_flow_integrate(self.h, flow, T, alpha, scheme, t, dt, _ptr(x), x.shape[1], _ptr(out),
                                     _stream(x.device)), "cmm_flow_integrate")
        return out

    def flow_advect_project(self, flow, scheme, t, dt, s_pts, tan, prev_coeffs, T=1.0, alpha=0.0,
                            eps=1e-5, jets=None, work=None):
        """One CMM map update under an analytic flow; returns (jets, work)."""
        s_pts, tan = _dev(s_pts), _dev(tan)
        if jets is None:
            jets = torch.empty((3, 4, self.nv), dtype=torch.float64, device=s_pts.device)
        if work is None:
            work = torch.empty(lib.cmm_advect_workspace(self.h), dtype=torch.float64, device=s_pts.device)
        check(lib.cmm_flow_advect_project(self.h, flow, T, alpha, scheme, t, dt, _ptr(s_pts), _ptr(tan),
                                          _ptr(prev_coeffs), eps, _ptr(jets), _ptr(work),
                                          _stream(s_pts.device)), "cmm_flow_advect_project")
        return jets, work

    def tracer(self, kind, X, t=0.0, out=None):
        """Tracer field at points X (n,3) -> (n,)."""
        X = _dev(X)
        n = X.shape[0]
        out = torch.empty(n, dtype=torch.float64, device=X.device) if out is None else out
        check(lib.cmm_tracer_eval(self.h, kind, t, _ptr(X), n, _ptr(out), _stream(X.device)),
              "cmm_tracer_eval")
        return out


EULER, IMPROVED_EULER, RK4, RK2 = 0, 1, 2, 3
(FLOW_SOLID_BODY, FLOW_DEFORM, FLOW_DEFORM_ROT, FLOW_STATIC_VORTEX, FLOW_ROTATING_VORTEX,
 FLOW_EQUATOR_VORTEX, FLOW_DIVERGENT) = range(7)
(TRACER_COSINE_BELL, TRACER_SLOTTED_CYLINDERS, TRACER_STATIC_VORTEX, TRACER_ROTATING_VORTEX,
 TRACER_SMOOTH_TEST, TRACER_RANDOM_SH) = range(6)
(VORT_NONE, VORT_ROSSBY_HAURWITZ, VORT_ZONAL_JET, VORT_PERTURBED_JET, VORT_MULTI_JET,
 VORT_GAUSSIAN_VORTEX, VORT_GAUSSIAN_JETS, VORT_PERTURBED_RH) = range(8)


class VelMesh(Mesh):
    """Device context of the MWSS lat-lon velocity mesh (cmm_velmesh_create)."""

    def __init__(self, L, theta, phi, grid, verts, device=None):  # noqa: super not called
        theta = np.ascontiguousarray(theta, dtype=np.float64)
        phi = np.ascontiguousarray(phi, dtype=np.float64)
        grid = np.ascontiguousarray(np.asarray(grid, dtype=np.float64).reshape(3, -1))
        verts = np.ascontiguousarray(verts, dtype=np.float64)
        self.device = torch.device("cuda", torch.cuda.current_device() if device is None else device)
        self.L, self.nv, self.level = L, len(verts), -1
        self.nt = 4 * L * (L - 1)
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            check(lib.cmm_velmesh_create(L, theta.ctypes.data, phi.ctypes.data, grid.ctypes.data,
                                         verts.ctypes.data, ctypes.byref(h)), "cmm_velmesh_create")
        self.h = h
        self.stride = lib.cmm_coeff_stride(3)

    REC_FP64, REC_FP32, REC_MIXED = 0, 1, 2

    def set_records(self, precision):
        """Velocity coefficient records in FP64 (default) or FP32
        (cmm_velmesh_set_records)."""
        with torch.cuda.device(self.device):
            check(lib.cmm_velmesh_set_records(self.h, precision), "cmm_velmesh_set_records")
        self.rec32 = precision != self.REC_FP64
        return self

    def new_coeffs(self, ncomp=3, batch=()):
        dt = torch.float32 if (ncomp == 3 and getattr(self, "rec32", False)) else torch.float64
        return torch.zeros((*batch, self.nt, lib.cmm_coeff_stride(ncomp)), dtype=dt, device=self.device)

    def vorticity(self, kind, params, X, rot_rate, sh=None, omega=None, spline=None):
        """omega (L+1, 2L) at the back-traced sample points X (Q,3)."""
        X = _dev(X)
        params = np.ascontiguousarray(params if params is not None else [], dtype=np.float64)
        if omega is None:
            omega = torch.empty((self.L + 1, 2 * self.L), dtype=torch.float64, device=X.device)
        lmax = -1 if sh is None else sh.shape[0] - 1
        check(lib.cmm_vorticity_eval(self.h, kind, params.ctypes.data if len(params) else None,
                                     len(params), _ptr(sh), lmax, _ptr(spline), rot_rate, _ptr(X),
                                     _ptr(omega), _stream(X.device)), "cmm_vorticity_eval")
        return omega

    def velocity(self, vel_coeffs, ts0, t, dt, x):
        x = _dev(x)
        out = torch.empty_like(x)
        arr = (ctypes.c_void_p * len(vel_coeffs))(*[c.data_ptr() for c in vel_coeffs])
        check(lib.cmm_velocity_eval(self.h, arr, len(vel_coeffs), ts0, t, dt, _ptr(x), x.shape[1],
                                    _ptr(out), _stream(x.device)), "cmm_velocity_eval")
        return out

    def integrate(self, vel_coeffs, ts0, scheme, t, dt, x):
        x = _dev(x)
        out = torch.empty_like(x)
        arr = (ctypes.c_void_p * len(vel_coeffs))(*[c.data_ptr() for c in vel_coeffs])
        check(lib.cmm_integrate(self.h, arr, len(vel_coeffs), ts0, scheme, t, dt, _ptr(x), x.shape[1],
                                _ptr(out), _stream(x.device)), "cmm_integrate")
        return out


class Sht:
    """MWSS transform plan at band-limit L (cmm_sht_create).

    Coefficients are complex128 tensors (L, L) indexed [m, l] (m <= l)."""

    def __init__(self, L, device=None):
        self.L = L
        self.device = torch.device("cuda", torch.cuda.current_device() if device is None else device)
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            check(lib.cmm_sht_create(L, ctypes.byref(h)), "cmm_sht_create")
        self.h = h

    def __del__(self):
        h = getattr(self, "h", None)
        if h is not None and h.value:
            lib.cmm_sht_destroy(h)
            self.h = None

    FP64, SPLIT_BF16 = 0, 1

    def set_precision(self, mode):
        with torch.cuda.device(self.device):
            check(lib.cmm_sht_set_precision(self.h, mode), "cmm_sht_set_precision")
        return self

    SCHEDULE_PER_CHUNK, SCHEDULE_WARP_SPECIALISED = 0, 1

    def set_schedule(self, schedule):
        """Split-BF16 synthesis schedule (cmm_sht_set_schedule)."""
        check(lib.cmm_sht_set_schedule(self.h, schedule), "cmm_sht_set_schedule")
        return self

    def share_tables(self, src):
        """Share src's Legendre tables (cmm_sht_share_tables): split-BF16
        mode on src's tables when src is in that mode, else src's FP64 Pbar
        tables."""
        with torch.cuda.device(self.device):
            check(lib.cmm_sht_share_tables(self.h, src.h), "cmm_sht_share_tables")
        self._tables_from = src   # keep the owner alive
        return self

    def trim(self):
        check(lib.cmm_sht_trim(self.h), "cmm_sht_trim")
        return self

    def timeout_selftest(self, polls=1000):
        """Make the bounded tensor-core wait run out (cmm_sht_timeout_selftest)."""
        check(lib.cmm_sht_timeout_selftest(self.h, int(polls), _stream(self.device)), "cmm_sht_timeout_selftest")
        return self

    TABLES_AUTO, TABLES_ALWAYS, TABLES_NEVER = 0, 1, -1

    def set_tables(self, mode):
        """FP64 Legendre stages from Pbar tables (cmm_sht_set_tables)."""
        with torch.cuda.device(self.device):
            check(lib.cmm_sht_set_tables(self.h, int(mode)), "cmm_sht_set_tables")
        return self

    def status(self, clear=True):
        f = ctypes.c_int()
        check(lib.cmm_sht_status(self.h, _stream(self.device), ctypes.byref(f), int(clear)),
              "cmm_sht_status")
        return f.value

    def forward(self, samples):
        samples = _dev(samples)
        alm = torch.zeros((self.L, self.L), dtype=torch.complex128, device=samples.device)
        check(lib.cmm_sht_forward(self.h, _ptr(samples), _ptr(alm), _stream(samples.device)),
              "cmm_sht_forward")
        return alm

    def inverse(self, alm):
        alm = _dev(alm, torch.complex128)
        nf = 1 if alm.dim() == 2 else alm.shape[0]
        out = torch.empty((nf, self.L + 1, 2 * self.L), dtype=torch.float64, device=alm.device)
        check(lib.cmm_sht_inverse(self.h, _ptr(alm), nf, _ptr(out), _stream(alm.device)),
              "cmm_sht_inverse")
        return out[0] if alm.dim() == 2 else out

    def power(self, alm):
        """Angular power per degree, sum over m = -l..l of |a_lm|^2 (L,)."""
        alm = _dev(alm, torch.complex128)
        out = torch.empty(self.L, dtype=torch.float64, device=alm.device)
        check(lib.cmm_sht_power(self.h, _ptr(alm), _ptr(out), _stream(alm.device)), "cmm_sht_power")
        return out

    def scalar_jets(self, velmesh, alm, jets=None):
        """Scalar jets (4, Nv_u) of the field with coefficients alm [m,l]."""
        alm = _dev(alm, torch.complex128)
        if jets is None:
            jets = torch.empty((4, velmesh.nv), dtype=torch.float64, device=alm.device)
        check(lib.cmm_sht_scalar_jets(self.h, velmesh.h, _ptr(alm), _ptr(jets), _stream(alm.device)),
              "cmm_sht_scalar_jets")
        return jets

    def velocity(self, velmesh, omega, jets=None, psi=None):
        omega = _dev(omega)
        if jets is None:
            jets = torch.empty((3, 4, velmesh.nv), dtype=torch.float64, device=omega.device)
        check(lib.cmm_sht_velocity(self.h, velmesh.h, _ptr(omega), _ptr(psi), _ptr(jets),
                                   _stream(omega.device)), "cmm_sht_velocity")
        return jets


class ShtBatch:
    """Split-BF16 plans of one band-limit whose forward analyses run as one
    tensor-core launch (cmm_sht_batch_create); holds its plans, so they
    outlive it."""
    MAX = 8

    def __init__(self, plans):
        self.plans = list(plans)
        self.device = self.plans[0].device
        arr = (ctypes.c_void_p * len(self.plans))(*[p.h.value for p in self.plans])
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            check(lib.cmm_sht_batch_create(arr, len(self.plans), ctypes.byref(h)), "cmm_sht_batch_create")
        self.h = h

    def __del__(self):
        h = getattr(self, "h", None)
        if h is not None and h.value:
            lib.cmm_sht_batch_destroy(h)
            self.h = None

    def analysis(self, stream=None):
        check(lib.cmm_sht_batch_analysis(self.h, stream if stream is not None else _stream(self.device)),
              "cmm_sht_batch_analysis")

    def forward(self, samples):
        """Forward transforms of one field per member (cmm_sht_batch_forward):
        samples[b] (L+1, 2L) -> alm[b] (L, L) complex128."""
        samples = [_dev(x) for x in samples]
        L = self.plans[0].L
        alm = [torch.zeros((L, L), dtype=torch.complex128, device=self.device) for _ in samples]
        sa = (ctypes.c_void_p * len(samples))(*[x.data_ptr() for x in samples])
        aa = (ctypes.c_void_p * len(alm))(*[a.data_ptr() for a in alm])
        check(lib.cmm_sht_batch_forward(self.h, sa, aa, _stream(self.device)), "cmm_sht_batch_forward")
        return alm


def compose_host(mesh, coeffs, q_host, out_host, tri_host=None, jac_host=None, chunks=8,
                 streams=None, scratch=None, order=None, forms=None, forms_ff=None, nstreams=4):
    """Composition of host-resident queries (pinned (n,3) float64) into
    host-resident outputs, pipelined in `chunks` pieces over `nstreams` CUDA
    streams (each with its own device buffers) so the host<->device copies
    overlap the kernels (2^24 queries with Jacobians through 8 submaps:
    12.8 ms with 8 chunks on 4 streams, 15.0 ms with 16 on 2).  order: each
    chunk is processed grouped by coarse cell (cmm_query_order, same
    results; default), so that neighbouring threads gather neighbouring
    records.  forms / forms_ff: map-form records and their float-float
    copies (Mesh.compose).  Returns the scratch dict for reuse."""
    if order is None:
        order = True
    n = q_host.shape[0]
    dev = mesh.device
    streams = streams or [torch.cuda.Stream(dev) for _ in range(nstreams)]
    step = (n + chunks - 1) // chunks
    if scratch is None:
        scratch = {}
        for k in range(len(streams)):
            scratch[k] = dict(
                q=torch.empty((step, 3), dtype=torch.float64, device=dev),
                out=torch.empty((step, 3), dtype=torch.float64, device=dev),
                tri=torch.empty(step, dtype=torch.int32, device=dev) if tri_host is not None else None,
                jac=torch.empty((step, 3, 3), dtype=torch.float64, device=dev) if jac_host is not None else None,
                perm=torch.empty(step, dtype=torch.int32, device=dev),
                work=torch.empty(lib.cmm_query_order_workspace(step), dtype=torch.int32, device=dev))
    arr = (ctypes.c_void_p * len(coeffs))(*[c.data_ptr() for c in coeffs])
    farr = None if forms is None else (ctypes.c_void_p * len(coeffs))(
        *[None if f is None else f.data_ptr() for f in forms])
    garr = None if forms_ff is None else (ctypes.c_void_p * len(coeffs))(
        *[None if g is None else g.data_ptr() for g in forms_ff])
    cur = torch.cuda.current_stream(dev)
    for s in streams:
        s.wait_stream(cur)
    for c in range(chunks):
        lo, hi = c * step, min(n, (c + 1) * step)
        if lo >= hi:
            break
        k = c % len(streams)
        s, b = streams[k], scratch[k]
        m = hi - lo
        with torch.cuda.stream(s):
            b["q"][:m].copy_(q_host[lo:hi], non_blocking=True)
            st = ctypes.c_void_p(s.cuda_stream)
            if order:
                check(lib.cmm_query_order(mesh.h, _ptr(b["q"]), m, _ptr(b["perm"]), _ptr(b["work"]), st),
                      "cmm_query_order")
            if farr is not None:
                check(lib.cmm_compose_forms(mesh.h, arr, farr, garr, len(coeffs), _ptr(b["q"]), m,
                                            _ptr(b["perm"]) if order else None, _ptr(b["out"]), _ptr(b["tri"]),
                                            None, _ptr(b["jac"]), st), "cmm_compose_forms")
            elif order:
                check(lib.cmm_compose_ordered(mesh.h, arr, len(coeffs), _ptr(b["q"]), m, _ptr(b["perm"]),
                                              _ptr(b["out"]), _ptr(b["tri"]), None, _ptr(b["jac"]), st),
                      "cmm_compose_ordered")
            else:
                check(lib.cmm_compose(mesh.h, arr, len(coeffs), _ptr(b["q"]), m, _ptr(b["out"]),
                                      _ptr(b["tri"]), None, _ptr(b["jac"]), st), "cmm_compose")
            out_host[lo:hi].copy_(b["out"][:m], non_blocking=True)
            if tri_host is not None:
                tri_host[lo:hi].copy_(b["tri"][:m], non_blocking=True)
            if jac_host is not None:
                jac_host[lo:hi].copy_(b["jac"][:m], non_blocking=True)
    for s in streams:
        cur.wait_stream(s)
    return scratch, streams
