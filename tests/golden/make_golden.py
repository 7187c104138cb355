"""Generate the golden fixtures from the reference implementation itself.

Runs only where the reference checkout exists (``REF`` below).  The
reference's ``cmm_s2.core`` modules are imported unchanged with import shims
for packages that are absent here:

* ``np.VisibleDeprecationWarning`` (removed in numpy 2) and
  ``scipy.special.sph_harm`` (removed in scipy 1.18) aliases;
* empty ``igl``/``numba``/``pathos`` modules (imported, never called);
* ``stripy.sTriangulation``: returns its input points in input order (the
  reference reads only ``.points/.x/.y/.z``); for the icosahedral meshes the
  exact generated points are handed through so both sides see identical
  vertices;
* ``pyssht.sample_positions`` / ``elm2ind`` (MWSS positions, l*l+l+m) and,
  for the one barotropic-vorticity fixture, ``forward``/``inverse`` backed by
  the oracle's restated MWSS transform (pyssht itself is absent).

Outputs: ``tests/golden/*.npz`` (small; committed).
Usage: python tests/golden/make_golden.py            (every fixture but the
       large-level Qhull tables)
       python tests/golden/make_golden.py qhull 5 6 (Qhull-order location
       fixtures ``qhull_l5.npz``/``qhull_l6.npz``; the level-6 Delaunay build
       takes ~13 min of one core)
       python tests/golden/make_golden.py bve_l4      (the whole barotropic
       configuration, level 4 / L = 128 / 200 steps: ``bve_l4_L128.npz``)
"""
import os
import sys
import types

import numpy as np
import scipy.special

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = "/root/reference"
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "cmm-s2_gb300"))
sys.path.insert(0, REF)

from cmm_gpu.meshgen import icosahedral_mesh, random_sphere_points  # noqa: E402
from cmm_gpu.workloads import submap_stack  # noqa: E402
from oracle import sht as osht  # noqa: E402

# ----------------------------------------------------------------- shims
np.VisibleDeprecationWarning = np.exceptions.VisibleDeprecationWarning
if not hasattr(scipy.special, "sph_harm"):
    scipy.special.sph_harm = lambda m, l, phi, theta: scipy.special.sph_harm_y(l, m, theta, phi)
for _name in ["igl", "numba", "pathos", "pathos.multiprocessing"]:
    sys.modules[_name] = types.ModuleType(_name)
sys.modules["numba"].njit = lambda *a, **k: (lambda f: f)
sys.modules["pathos.multiprocessing"].ProcessingPool = object

_EXACT = {"pts": None}


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


_stripy = types.ModuleType("stripy")
_stripy.sTriangulation = _STri
sys.modules["stripy"] = _stripy
_pysh = types.ModuleType("pyssht")
_pysh.sample_positions = lambda L, Method="MWSS", Grid=False: (np.pi * np.arange(L + 1) / L,
                                                               2 * np.pi * np.arange(2 * L) / (2 * L))
_pysh.elm2ind = lambda l, m: l * l + l + m
_SHT = {}


def _sht(L):
    if L not in _SHT:
        _SHT[L] = osht.MWSS(L)
    return _SHT[L]


def _forward(f, L, Spin=0, Method="MWSS", Reality=True, backend=None, nthreads=1):
    return osht.full_from_half(_sht(L).forward(np.real(f)))


def _inverse(flm, L, Spin=0, Method="MWSS", Reality=True, backend=None, nthreads=1):
    return _sht(L).inverse(osht.half_from_full(flm, L))


_pysh.forward, _pysh.inverse = _forward, _inverse
sys.modules["pyssht"] = _pysh

from cmm_s2.core import mesh_functions as rmesh  # noqa: E402
from cmm_s2.core import spherical_spline as rspl  # noqa: E402
from cmm_s2.core import evolution_functions as revol  # noqa: E402
from cmm_s2.core import spherical_harmonic_tools as rsht  # noqa: E402
from cmm_s2.core import spherical_simulations as rsim  # noqa: E402
from cmm_s2.core import dynamical_fields as rfields  # noqa: E402
from cmm_s2.core import utils as rutils  # noqa: E402


def ref_mesh(level):
    verts, _ = icosahedral_mesh(level)
    _EXACT["pts"] = verts
    m = rmesh.spherical_triangulation(verts)
    _EXACT["pts"] = None
    assert np.array_equal(m.vertices, verts)
    return m


def special_points(verts, tris):
    """Vertices, edge midpoints, centroids and poles: exact-tie cases."""
    v = verts[tris[:64]]
    mids = (v[:, 0] + v[:, 1]) / np.linalg.norm(v[:, 0] + v[:, 1], axis=1)[:, None]
    cent = v.sum(1) / np.linalg.norm(v.sum(1), axis=1)[:, None]
    return np.concatenate([verts[:32], mids, cent, [[0, 0, 1.0], [0, 0, -1.0], [1.0, 0, 0]]])


def save(name, **arrays):
    path = os.path.join(HERE, name)
    np.savez_compressed(path, **arrays)
    print("wrote", path, sum(a.nbytes for a in map(np.asarray, arrays.values())) // 1024, "KiB raw")


def qhull_fixture(level, nq=16384):
    """Qhull-order triangle table and ``find_simplex`` ids at a large level.

    The reference's triangle index is the row of Qhull's Delaunay simplex
    table (cmm_s2/core/mesh_functions.py:43-56, 82).  Stored: that table,
    the ids and barycentrics of ``nq`` seeded random queries plus the exact
    tie points; the vertices and the random queries are regenerated by the
    test from ``icosahedral_mesh(level)`` and ``random_sphere_points(nq,
    seed)``, with SHA-256 digests to prove they are the same bytes.
    """
    import hashlib
    import time
    t0 = time.time()
    m = ref_mesh(level)
    t1 = time.time()
    tris = np.asarray(m.simplices)
    seed = 50 + level
    qr = random_sphere_points(nq, seed=seed)
    qs = special_points(m.vertices, tris)
    q = np.concatenate([qr, qs])
    bcc, tri, _ = m.query(q)
    print(f"level {level}: Delaunay {t1 - t0:.0f} s, query {time.time() - t1:.1f} s")
    save(f"qhull_l{level}.npz", tris=tris.astype(np.int32), seed=seed, nq=nq, q_special=qs,
         tri=tri.astype(np.int32), bcc=bcc,
         verts_sha=hashlib.sha256(np.ascontiguousarray(m.vertices).tobytes()).hexdigest(),
         q_sha=hashlib.sha256(np.ascontiguousarray(qr).tobytes()).hexdigest())


def bve_level4_L128(nq=2000):
    """The barotropic configuration run in full by the reference driver
    (euler_simulation_sphere_remapping, cmm_s2/core/spherical_simulations.py:
    144-297): level-4 mesh, L = 128, T = 1 in 200 steps (dt = 1/200),
    n_maps = 20 (remap every 20 steps, 10 submaps), rotation 2 pi; initial
    vorticity the real SH series of degrees 1..16 with N(0,1) l^-1.5
    coefficients from seed 0 (cmm_gpu.workloads.random_sh_vorticity).  The
    restated MWSS transform stands in for pyssht.  Stored: the final
    composite map at nq seeded random points and the vorticity there
    (omega0(X) + 2 Omega cos theta(X) - 2 Omega cos theta); and the same
    from the oracle's run of the configuration with the closed-form
    sub-triangle barycentrics (``img_closed``/``omega_closed``), whose
    difference from the reference's run is the reference's own
    finite-difference noise floor."""
    import time
    from cmm_gpu.workloads import random_sh_vorticity
    omega0, a = random_sh_vorticity(16, seed=0)
    m = ref_mesh(4)
    t0 = time.time()
    subs = rsim.euler_simulation_sphere_remapping(128, 200, 1.0, m, omega0, rot_rate=2 * np.pi, n_maps=20)
    print(f"level-4 / L=128 run {time.time() - t0:.0f} s")
    q = random_sphere_points(nq, seed=123)
    img = subs(q.copy())
    phi, theta = rutils.cart2sphere(img.T)
    _, theta_q = rutils.cart2sphere(q.T)
    om = omega0(phi, theta) + 4 * np.pi * np.cos(theta) - 4 * np.pi * np.cos(theta_q)
    from oracle.bve import BVEOracle
    from oracle import geometry as OG
    tris = np.asarray(m.simplices)
    t0 = time.time()
    orc = BVEOracle(m.vertices, tris, OG.ConeLocator(m.vertices, tris), 128, 200, 1.0, omega0, n_maps=20,
                    closed=True, tie_fix=True).run()
    print(f"oracle closed-form run {time.time() - t0:.0f} s")
    imgc = orc.composite()(q)
    phc, thc = rutils.cart2sphere(imgc.T)
    omc = omega0(phc, thc) + 4 * np.pi * np.cos(thc) - 4 * np.pi * np.cos(theta_q)
    save("bve_l4_L128.npz", q=q, img=img, omega=om, img_closed=imgc, omega_closed=omc, Nc=subs.Nc,
         ns=np.array(subs.ns), sh=a)


def main():
    # ---- icosahedral meshes, query, PS maps, composite --------------------
    for level in (3, 4):
        m = ref_mesh(level)
        tris = np.asarray(m.simplices)
        q = np.concatenate([random_sphere_points(3000, seed=10 + level), special_points(m.vertices, tris)])
        bcc, tri, _ = m.query(q)
        Hs, Gs, Es = m.ps_split
        if level != 3:
            save(f"mesh_l{level}.npz", verts=m.vertices, tris=tris.astype(np.int32), q=q, bcc=bcc,
                 tri=tri.astype(np.int32))
            continue
        save(f"mesh_l{level}.npz", verts=m.vertices, tris=tris.astype(np.int32),
             H=np.stack([h.T for h in Hs]), G=np.stack(Gs), E=np.stack(Es),
             tan=np.stack(m.tan_vects), s_pts=m.s_pts, q=q, bcc=bcc, tri=tri.astype(np.int32))
        jets = submap_stack(m.s_pts, np.stack(m.tan_vects), 3, seed=5)
        nt = len(tris)
        mp = rspl.sphere_diffeomorphism(m, jets[0].copy(), np.zeros((3, 19, nt)))
        img = mp(q)
        # stencil evaluation: vertex foot points yn and stencil foot points
        rng = np.random.default_rng(3)
        rot = np.linalg.qr(rng.standard_normal((3, 3)))[0]
        rot *= np.sign(np.linalg.det(rot))
        yn = (m.vertices @ rot.T).T
        sp = np.einsum("ij,jkn->ikn", rot, m.s_pts)
        st = mp.stencil_eval(yn.copy(), sp.copy())
        comp = rspl.composite_sphere_diffeomorphism(m, jets.copy(), np.zeros((3, 3, 19, nt)), [1, 2, 3])
        for i in range(3):
            comp.assemble_coefficients(i, jets[i].copy())
        comp.Nc = 3
        cimg = comp(q.copy())
        save("map_l3.npz", jets=jets, coeffs0=mp.coeffs, q=q, img=img, yn=yn, sp=sp, st=st, comp_img=cimg)

        # ---- one CMM update: advect + project (RK4 and Euler), L=8 velocity
        L = 8
        mu = rmesh.structure_spherical_triangulation(L)
        ntu = len(mu.simplices)
        vals_u = np.zeros((3, 3, 4, len(mu.vertices)))
        U = rspl.spline_interp_velocity(mu, vals_u, np.zeros((3, 3, 19, ntu)), ts=np.array([0.0, 0.1, 0.2]))
        Phi, The = np.meshgrid(mu.phi, mu.theta)
        dinv = osht.inverse_laplacian_diag(L)
        lp, lmn, lz = osht.ladder_operators(L)
        for n, t in enumerate([0.0, 0.1, 0.2]):
            om = rfields.rossby_wave(Phi, The, t=t) + 0.3 * np.sin(The) ** 2 * np.cos(2 * Phi + t)
            psi = rsht.inv_Laplacian(om, L, dinv)
            rsht.project_stream(psi, L, lp, lmn, lz, U, n, 0 * psi)
        U.nVs = 3
        qv = np.concatenate([random_sphere_points(2000, seed=21), special_points(m.vertices, tris),
                             np.array(mu.grid_points).reshape(3, -1).T[:40]])
        bcc_u, tri_u, _ = mu.query(qv)
        vel = U(0.23, 0.1, qv.T.copy())
        save("velocity_L8.npz", vals=U.vals, coeffs=U.coeffs, verts=mu.vertices,
             simplices=np.asarray(mu.simplices), msimplices=mu.msimplices, q=qv, bcc=bcc_u,
             tri=tri_u, t=0.23, dt=0.1, ts=np.array([0.0, 0.1, 0.2]), vel=vel)
        map0 = rspl.sphere_diffeomorphism(m, jets[0].copy(), np.zeros((3, 19, nt)))
        new_rk4 = revol.advect_project_sphere(map0, revol.RK4_proj, 0.05, 0.1, U, identity=False)
        map1 = rspl.sphere_diffeomorphism(m, jets[1].copy(), np.zeros((3, 19, nt)))
        U.nVs = 1
        new_eul = revol.advect_project_sphere(map1, revol.Euler_step_proj, 0.0, 0.1, U, identity=True)
        U.nVs = 2
        new_ie = revol.advect_project_sphere(map1, revol.improved_Euler_proj, 0.0, 0.1, U, identity=True)
        save("advect_l3_L8.npz", jets_prev=jets[0], jets_rk4=new_rk4.vals, jets_euler=new_eul.vals,
             jets_ieuler=new_ie.vals)

    # ---- coefficient-space operators ----------------------------------------
    L = 8
    rng = np.random.default_rng(7)
    flm = rng.standard_normal(L * L) + 1j * rng.standard_normal(L * L)
    ca = rsht.coeff_array(flm, L)
    lp, lmn, lz = osht.ladder_operators(L)
    am = rsht.angular_momentum(ca, lp, lmn, lz, 0 * ca)
    save("sht_ops_L8.npz", flm=flm, coeff_array=ca, lm_array=rsht.lm_array(ca, L), ang_x=am[0],
         ang_y=am[1], ang_z=am[2])

    # ---- scalar spline of a spherical-harmonic field (project_onto_S12) -----
    L = 8
    mu = rmesh.structure_spherical_triangulation(L)
    alms = np.zeros((L, 2 * L + 1), dtype=complex)
    rng = np.random.default_rng(11)
    half = np.tril(rng.standard_normal((L, L)) + 1j * rng.standard_normal((L, L)))
    half[:, 0] = half[:, 0].real
    alms[:] = osht.shifted_from_vec(osht.full_from_half(half), L)
    sp = rsht.project_onto_S12(alms, L, mu)
    ph = np.linspace(0.1, 6.2, 23)
    th = np.linspace(0.05, 3.1, 19)
    PH, TH = np.meshgrid(ph, th)
    save("scalar_L8.npz", alm_half=half, vals=sp.vals, coeffs=sp.coeffs, phi=PH, theta=TH,
         value=sp(PH.copy(), TH.copy()))

    # ---- initial vorticity fields at scattered points ----------------------
    Xf = random_sphere_points(400, seed=41)
    phi, theta = rutils.cart2sphere(Xf.T)
    fields = dict(X=Xf, rossby_wave=rfields.rossby_wave(phi, theta, t=0.3), zonal_jet=rfields.zonal_jet(phi, theta),
                  perturbed_zonal_jet=rfields.perturbed_zonal_jet(phi, theta),
                  multi_jet=rfields.multi_jet(phi, theta), gaussian_vortex=rfields.gaussian_vortex(phi, theta),
                  perturbed_rossby_wave=rfields.perturbed_rossby_wave(phi, theta),
                  rotating_frame=rfields.rotating_frame(phi, theta))
    save("fields.npz", **fields)

    # ---- linear transport: analytic flows, tracers, a remapped run ----------
    m = ref_mesh(3)
    tris = np.asarray(m.simplices)
    X = np.concatenate([random_sphere_points(600, seed=31), special_points(m.vertices, tris),
                        [[0, 0, 1.0], [0, 0, -1.0], [0, 1.0, 0], [-1.0, 0, 0]]])
    flows = ["u_sbr", "u_deform", "u_deform_rot", "u_static_vortex", "u_rotating_vortex", "equator_vortex",
             "u_div"]
    out = dict(X=X)
    for name in flows:
        for k, t in enumerate([0.0, 0.37]):
            out[f"vel_{name}_{k}"] = np.asarray(getattr(rfields, name)(t, 0.05, X.T.copy()))
    phi, theta = rutils.cart2sphere(X.T)
    out["tr_cosine_bell"] = rfields.cosine_bell(phi, theta)
    out["tr_IC_SC"] = rfields.IC_SC(phi, theta)
    out["tr_static_vort_IC"] = rfields.static_vort_IC(0.4, X.T.copy())
    out["tr_rotating_vort_IC"] = rfields.rotating_vort_IC(0.4, X.T.copy())
    out["tr_random_initial_condition"] = rfields.random_initial_condition(X.T.copy())
    # the loop of tests/test_spherical_transport.py at level 3 (Nt = 2^3 + 10
    # steps of RK4 over T = 1, u_deform_rot) with remapping every 5 steps
    verts = m.vertices
    jet0 = np.zeros((3, 4, len(verts)))
    jet0[:, 0, :] = verts.T
    jet0[:, 1:, :] = np.array([rutils.grad_x(verts.T), rutils.grad_y(verts.T), rutils.grad_z(verts.T)])
    nt = len(tris)
    map0 = rspl.sphere_diffeomorphism(m, jet0.copy(), np.zeros((3, 19, nt)))
    Nt = 2 ** 3 + 10
    tspan = np.linspace(0, 1, Nt, endpoint=False)
    dt = tspan[1] - tspan[0]
    remaps, mapping, identity = [], map0, True
    for count, t in enumerate(tspan, start=1):
        mapping = revol.advect_project_sphere(mapping, revol.RK4_proj, t, dt, rfields.u_deform_rot, identity)
        identity = False
        if count % 5 == 0:
            remaps.append(mapping.vals.copy())
            mapping = rspl.sphere_diffeomorphism(m, jet0.copy(), np.zeros((3, 19, nt)))
            identity = True
    if not identity:
        remaps.append(mapping.vals.copy())
    q = random_sphere_points(400, seed=32)
    ev = q.copy()
    for vals in remaps[::-1]:
        ev = rspl.sphere_diffeomorphism(m, vals.copy(), np.zeros((3, 19, nt)))(ev.copy()).T
    out.update(jet0=jet0, remaps=np.stack(remaps), q=q, evals=ev, dt=dt, Nt=Nt)
    # one RK2 step of the solid-body rotation from the identity
    rk2 = revol.advect_project_sphere(map0, revol.RK2_proj, 0.0, 0.05, rfields.u_sbr, True)
    out["jets_rk2_sbr"] = rk2.vals
    save("transport_l3.npz", **out)

    # ---- a short barotropic run (restated transforms stand in for pyssht) ---
    m2 = ref_mesh(2)
    subs = rsim.euler_simulation_sphere_remapping(8, 12, 1.0, m2, rfields.rossby_wave,
                                                  rot_rate=2 * np.pi, n_maps=5)
    qe = random_sphere_points(500, seed=99)
    save("bve_l2_L8.npz", vals=subs.vals[:subs.Nc], Nc=subs.Nc, ns=np.array(subs.ns), q=qe, img=subs(qe.copy()))

    # ---- the reference's own files: the video driver's snapshot pickles and
    # its pickled submap stack (read back by cmm_gpu.state_io)
    import shutil
    import tempfile
    tmp = tempfile.mkdtemp()
    try:
        rsim.euler_simulation_sphere_remapping_video(8, 12, 1.0, m2, rfields.rossby_wave, 2 * np.pi, 5,
                                                     os.path.join(tmp, "run"), 3)
        for name in sorted(os.listdir(tmp)):
            shutil.copy(os.path.join(tmp, name), os.path.join(HERE, "ref_video_l2_" + name.replace(".txt", ".pkl")))
            print("wrote", os.path.join(HERE, "ref_video_l2_" + name.replace(".txt", ".pkl")))
    finally:
        shutil.rmtree(tmp)


if __name__ == "__main__":
    if len(sys.argv) > 1 and sys.argv[1] == "qhull":
        for lv in sys.argv[2:]:
            qhull_fixture(int(lv))
    elif len(sys.argv) > 1 and sys.argv[1] == "bve_l4":
        bve_level4_L128()
    else:
        main()
