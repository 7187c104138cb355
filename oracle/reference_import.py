"""The reference implementation itself, imported unchanged for the reference
arm of bench.py (and by the fixture generator).  Test infrastructure only:
nothing in the library imports it.

seth-tl/CMM-S2 is pure Python (numpy/scipy) whose modules import
third-party packages that are not installed.  They are
replaced by shims at import time, none of which is on the timed map path
except through data it reads:

* ``np.VisibleDeprecationWarning`` (removed in numpy 2) and
  ``scipy.special.sph_harm`` (removed in scipy 1.18) aliases;
* empty ``igl``/``numba``/``pathos`` modules (imported, never called on the
  path);
* ``stripy.sTriangulation``: returns its input points in input order (the
  reference reads only ``.points/.x/.y/.z``,
  cmm_s2/core/mesh_functions.py:39, 61); the exact icosahedral vertices are
  handed through (``exact_points``) so both sides see identical vertices;
* ``pyssht.sample_positions`` / ``elm2ind`` (MWSS positions, l*l+l+m) and,
  when a transform is given, ``forward``/``inverse`` (pyssht itself is
  absent; the oracle's restated MWSS transform stands in).

Where the code comes from: ``copy_reference()`` copies the reference's
``cmm_s2`` package sources (``core`` and the package ``__init__``) into
``baseline/_ref/`` (git-ignored; it travels with the repository snapshot to
machines where the reference checkout does not exist);
``import_core()`` imports from that copy.
"""
import os
import shutil
import sys
import types

import numpy as np
import scipy.special

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_DIR = os.path.join(ROOT, "baseline", "_ref")
REF_CHECKOUT = "/root/reference"

_EXACT = {"pts": None}


def copy_reference(src=REF_CHECKOUT, dst=REF_DIR):
    """Copy the reference's cmm_s2 package (its __init__ and core/*.py)
    into dst; a no-op when the checkout is absent or the copy exists.
    Returns True when dst holds the package afterwards."""
    pkg = os.path.join(dst, "cmm_s2")
    if not os.path.exists(os.path.join(pkg, "core", "spherical_spline.py")) and \
            os.path.isdir(os.path.join(src, "cmm_s2", "core")):
        os.makedirs(os.path.join(pkg, "core"), exist_ok=True)
        shutil.copy(os.path.join(src, "cmm_s2", "__init__.py"), os.path.join(pkg, "__init__.py"))
        for name in os.listdir(os.path.join(src, "cmm_s2", "core")):
            if name.endswith(".py"):
                shutil.copy(os.path.join(src, "cmm_s2", "core", name), os.path.join(pkg, "core", name))
    return os.path.exists(os.path.join(pkg, "core", "spherical_spline.py"))


class _STri:
    def __init__(self, lons, lats, refinement_levels=0, permute=False, tree=False):
        lons = np.asarray(lons, dtype=np.float64)
        lats = np.asarray(lats, dtype=np.float64)
        if _EXACT["pts"] is not None and len(_EXACT["pts"]) == len(lons):
            p = _EXACT["pts"]
            self.x, self.y, self.z = p[:, 0].copy(), p[:, 1].copy(), p[:, 2].copy()
        else:
            self.x = np.cos(lats) * np.cos(lons)
            self.y = np.cos(lats) * np.sin(lons)
            self.z = np.sin(lats)
        self.points = np.stack([self.x, self.y, self.z], 1)


def install_shims(forward=None, inverse=None):
    """Register the stand-in modules (idempotent).  forward/inverse: the
    pyssht.forward/inverse replacements, when the caller needs transforms."""
    np.VisibleDeprecationWarning = np.exceptions.VisibleDeprecationWarning
    if not hasattr(scipy.special, "sph_harm"):
        scipy.special.sph_harm = lambda m, l, phi, theta: scipy.special.sph_harm_y(l, m, theta, phi)
    for name in ["igl", "numba", "pathos", "pathos.multiprocessing"]:
        if name not in sys.modules:
            sys.modules[name] = types.ModuleType(name)
    sys.modules["numba"].njit = lambda *a, **k: (lambda f: f)
    sys.modules["pathos.multiprocessing"].ProcessingPool = object
    if "stripy" not in sys.modules:
        st = types.ModuleType("stripy")
        st.sTriangulation = _STri
        sys.modules["stripy"] = st
    ps = sys.modules.get("pyssht") or types.ModuleType("pyssht")
    ps.sample_positions = lambda L, Method="MWSS", Grid=False: (np.pi * np.arange(L + 1) / L,
                                                                2 * np.pi * np.arange(2 * L) / (2 * L))
    ps.elm2ind = lambda l, m: l * l + l + m
    if forward is not None:
        ps.forward, ps.inverse = forward, inverse
    sys.modules["pyssht"] = ps


def import_core(path=None):
    """The reference's cmm_s2.core modules, imported from the copy under
    baseline/_ref (or `path`) behind the shims: a namespace with mesh_functions,
    spherical_spline, evolution_functions, utils."""
    path = path or REF_DIR
    if not os.path.exists(os.path.join(path, "cmm_s2", "core", "spherical_spline.py")):
        raise FileNotFoundError(f"the reference's sources are not under {path} (copy_reference)")
    install_shims()
    if path not in sys.path:
        sys.path.insert(0, path)
    import importlib
    mods = {n: importlib.import_module(f"cmm_s2.core.{n}")
            for n in ("utils", "mesh_functions", "spherical_spline", "evolution_functions")}
    return types.SimpleNamespace(**mods)


def mesh(core, verts):
    """The reference's spherical_triangulation (Qhull Delaunay of the
    vertices, cmm_s2/core/mesh_functions.py:29-66) of exactly `verts`."""
    _EXACT["pts"] = verts
    try:
        m = core.mesh_functions.spherical_triangulation(verts)
    finally:
        _EXACT["pts"] = None
    assert np.array_equal(m.vertices, verts)
    return m
