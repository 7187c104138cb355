"""GPU parity of whole barotropic-vorticity runs.

The reference rebuilds map gradients by centred differences with step
1e-5 of sub-triangle evaluations it computes from four fresh determinants
per point; their independent rounding, amplified 2.5e4 times, gives its
runs a noise floor: a run evaluated with the closed-form sub-triangle
barycentrics (the same linear maps, shared rounding) differs from the
reference's own run by ~2e-10 in map coordinates after 12 steps
(measured with the oracle in both forms).  So:
  * against the reference's golden run: within 5x that measured spread;
  * against the oracle in closed form: map coordinates within 1e-10 and
    vorticity within 1e-9 relative (the library and the oracle still
    round differently, ~1e-16 per operation, and the difference quotient
    amplifies that 2.5e4 times every step);
  * the Rossby-Haurwitz wave (an exact travelling solution) is reproduced
    with the oracle's error."""
import os

import numpy as np
import pytest
import torch

from conftest import GOLDEN
from oracle import geometry as OG
from oracle.bve import BVEOracle
from oracle.fields import rossby_wave

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sims():
    import __graft_entry__
    __graft_entry__.build()
    from cmm_gpu import spherical_simulations
    return spherical_simulations


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def test_short_run_matches_reference(sims):
    from cmm_gpu.meshgen import icosahedral_mesh
    d = np.load(os.path.join(GOLDEN, "bve_l2_L8.npz"))
    verts, _ = icosahedral_mesh(2)
    ql = OG.QhullLocator(verts)
    s = sims.BVESolver(verts, ql.tris, 2, 8, 12, 1.0, "rossby_wave", n_maps=5).run()
    assert s.Nc == int(d["Nc"]) and s.ns == list(d["ns"])
    img, _ = s.composite(dev(d["q"]))
    img = img.cpu().numpy()
    jets = np.stack([j.cpu().numpy() for j in s.stack_jets[:s.Nc]])
    orc = BVEOracle(verts, ql.tris, ql, 8, 12, 1.0, rossby_wave, n_maps=5, closed=True,
                    tie_fix=True).run()
    spread = np.abs(orc.composite()(d["q"]) - d["img"]).max()
    assert spread < 1e-9
    np.testing.assert_allclose(img, d["img"], rtol=0, atol=5 * spread + 1e-12)
    np.testing.assert_allclose(jets[:, :, 0], d["vals"][:, :, 0], rtol=0, atol=1e-9)
    np.testing.assert_allclose(img, orc.composite()(d["q"]), rtol=0, atol=1e-10)
    assert s.mesh.status() == 0 and s.vm.status() == 0


def test_level4_run_against_closed_form_oracle(sims):
    from cmm_gpu.meshgen import icosahedral_mesh, random_sphere_points
    verts, tris = icosahedral_mesh(4)
    q = random_sphere_points(2000, seed=4)
    s = sims.BVESolver(verts, tris, 4, 32, 30, 1.0, "rossby_wave", n_maps=10).run()
    orc = BVEOracle(verts, tris, OG.ConeLocator(verts, tris), 32, 30, 1.0, rossby_wave, n_maps=10,
                    closed=True, tie_fix=True).run()
    img = s.composite(dev(q))[0].cpu().numpy()
    np.testing.assert_allclose(img, orc.composite()(q), rtol=0, atol=1e-10)
    om = s.omega.cpu().numpy()
    np.testing.assert_allclose(om / np.abs(om).max(), orc.last_omega / np.abs(om).max(), rtol=0,
                               atol=1e-9)


def test_rossby_haurwitz_known_answer(sims):
    """cmm_s2/tests/test_barotropic_vorticity.py:40-43, 81-90: the wave
    travels exactly; compare omega(T) with rossby_wave(t=1)."""
    from cmm_gpu.meshgen import icosahedral_mesh
    verts, tris = icosahedral_mesh(3)
    L, Nt = 32, 2 ** 4 + 10
    s = sims.BVESolver(verts, tris, 3, L, Nt, 1.0, "rossby_wave", n_maps=10).run()
    n = 60
    ph, th = np.meshgrid(np.linspace(0, 2 * np.pi, n, endpoint=False), np.linspace(0, np.pi, n, endpoint=False))
    q = np.stack([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th)], -1).reshape(-1, 3)
    X = s.composite(dev(q))[0].cpu().numpy().T
    ang = OG.cart2sphere(X)
    Om = 2 * np.pi
    om = rossby_wave(ang[0], ang[1]) + 2 * Om * np.cos(ang[1]) - 2 * Om * np.cos(th.reshape(-1))
    err = np.abs(om - rossby_wave(ph.reshape(-1), th.reshape(-1), t=1)).max()
    orc = BVEOracle(verts, tris, OG.ConeLocator(verts, tris), L, Nt, 1.0, rossby_wave, n_maps=10,
                    closed=True, tie_fix=True).run()
    Xo = orc.composite()(q).T
    ango = OG.cart2sphere(Xo)
    omo = rossby_wave(ango[0], ango[1]) + 2 * Om * np.cos(ango[1]) - 2 * Om * np.cos(th.reshape(-1))
    erro = np.abs(omo - rossby_wave(ph.reshape(-1), th.reshape(-1), t=1)).max()
    print(f"RH L_inf error: gpu {err:.6e} oracle {erro:.6e}")
    assert err < 0.5 and abs(err - erro) < 1e-9


def test_diagnostics_rossby_haurwitz(sims):
    """Run diagnostics on the travelling Rossby-Haurwitz wave: the L_inf
    error on the MWSS grid against the exact solution, enstrophy and energy
    drift; the split-BF16 form's errors stay within 2x of the FP64 form's."""
    from cmm_gpu.meshgen import icosahedral_mesh
    verts, tris = icosahedral_mesh(4)
    L, Nt = 64, 42
    out = {}
    for form in ("fp64", "split_bf16"):
        s = sims.BVESolver(verts, tris, 4, L, Nt, 1.0, "rossby_wave", n_maps=10, precision=form).run()
        th, ph = np.meshgrid(np.pi * np.arange(L + 1) / L, np.pi * np.arange(2 * L) / L, indexing="ij")
        d = s.diagnostics(omega_true=rossby_wave(ph, th, t=1))
        print(form, d)
        out[form] = d
        assert d["linf_rel"] < 0.05
        assert d["enstrophy_drift"] < 1e-3 and d["energy_drift"] < 1e-3
    assert out["split_bf16"]["linf_rel"] < 2 * out["fp64"]["linf_rel"]
    assert out["split_bf16"]["enstrophy_drift"] < 2 * out["fp64"]["enstrophy_drift"] + 1e-6


def test_jacobian_determinant_converges(sims):
    """The back-to-label map is area preserving; its spline's tangent
    Jacobian determinant deviates from 1 by the interpolation error of the
    derivative, which must fall with mesh refinement (O(h^2): about 4x per
    level) on the Rossby-Haurwitz run."""
    from cmm_gpu.meshgen import icosahedral_mesh
    devs = []
    for level in (3, 4, 5):
        verts, tris = icosahedral_mesh(level)
        s = sims.BVESolver(verts, tris, level, 64, 42, 1.0, "rossby_wave", n_maps=10).run()
        devs.append(s.diagnostics(jacobian=True)["jac_det_dev"])
    print("max |det DX - 1| at levels 3, 4, 5:", devs)
    assert devs[1] < devs[0] / 2 and devs[2] < devs[1] / 2


def _small_solver(sims, precision="fp64"):
    from cmm_gpu.meshgen import icosahedral_mesh
    from cmm_gpu.workloads import random_sh_vorticity
    verts, tris = icosahedral_mesh(3)
    _, sh = random_sh_vorticity(8, seed=4)
    vort = sims.Vorticity("rossby_wave", (0.0,), sh=sh)
    return sims.BVESolver(verts, tris, 3, 16, 27, 1.0, vort, n_maps=5, precision=precision)


@pytest.mark.parametrize("precision", ["fp64", "split_bf16"])
def test_device_driven_step_matches_host_step(sims, precision):
    """cmm_bve_step (device-resident state, device bookkeeping, stage
    weights recomputed on the device) against the same run driven from the
    host through the single calls: bit-identical maps, stack and vorticity,
    including the remaps (n_maps = 5, Nt = 27: remaps at 5, 10, ..., 25, 27)."""
    a, b = _small_solver(sims, precision), _small_solver(sims, precision)
    a.bootstrap()
    b.bootstrap()
    for _ in range(a.Nt - 2):
        a.step()
        b.step_host()
    assert a.Nc == b.Nc == len(a.ns) and a.count == b.count == a.Nt
    for k in range(a.Nc):
        assert torch.equal(a.stack[k], b.stack[k]), k
        assert torch.equal(a.stack_jets[k], b.stack_jets[k]), k
    assert torch.equal(a.omega, b.omega)
    assert torch.equal(a.jets, b.jets)
    cnt, nc, ident = [ctypes_int() for _ in range(3)]
    from cmm_gpu import native
    native.check(native.lib.cmm_bve_state(a._bve, native._stream(), *(byref(x) for x in (cnt, nc, ident))),
                 "cmm_bve_state")
    assert (cnt.value, nc.value, ident.value) == (a.count, a.Nc, int(a.identity))
    assert a.mesh.status() == 0 and a.vm.status() == 0


@pytest.mark.parametrize("whole_run", [False, True])
def test_captured_graph_replays_the_run(sims, whole_run):
    """One step captured into a CUDA graph and replayed for every later
    step, or (whole_run) every remaining step captured into one graph and
    launched once, gives the run of the stepper called step by step, bit
    for bit."""
    a, b = _small_solver(sims), _small_solver(sims)
    a.bootstrap()
    b.bootstrap()
    n = a.Nt - 2
    b.capture(steps=n if whole_run else 1)
    for _ in range(n):
        a.step()
    for _ in range(1 if whole_run else n):
        b.step()
    torch.cuda.synchronize()
    assert (a.count, a.Nc, a.identity) == (b.count, b.Nc, b.identity)
    for k in range(a.Nc):
        assert torch.equal(a.stack[k], b.stack[k]), k
    assert torch.equal(a.omega, b.omega)
    q = torch.nn.functional.normalize(torch.randn(1000, 3, dtype=torch.float64, device="cuda"), dim=1)
    assert torch.equal(a.composite(q)[0], b.composite(q)[0])


def ctypes_int():
    import ctypes
    return ctypes.c_int()


def byref(x):
    import ctypes
    return ctypes.byref(x)


def test_vorticity_fields_match_reference(sims):
    """Every built-in initial-vorticity field at scattered points (with the
    planetary term off) against the reference's dynamical_fields values."""
    from cmm_gpu import native
    from cmm_gpu.meshgen import latlon_mesh_arrays
    d = np.load(os.path.join(GOLDEN, "fields.npz"))
    X = d["X"]
    L = 14                                  # (L+1) 2L = 420 >= 400 sample slots
    theta, phi, grid, vverts = latlon_mesh_arrays(L)
    vm = native.VelMesh(L, theta, phi, grid, vverts)
    Xp = np.concatenate([X, np.tile([[0.0, 0.0, 1.0]], ((L + 1) * 2 * L - len(X), 1))])
    cases = [(native.VORT_ROSSBY_HAURWITZ, [0.3], "rossby_wave"), (native.VORT_ZONAL_JET, [], "zonal_jet"),
             (native.VORT_PERTURBED_JET, [], "perturbed_zonal_jet"), (native.VORT_MULTI_JET, [], "multi_jet"),
             (native.VORT_GAUSSIAN_VORTEX, [], "gaussian_vortex"),
             (native.VORT_PERTURBED_RH, [], "perturbed_rossby_wave")]
    for kind, params, name in cases:
        om = vm.vorticity(kind, params, dev(Xp), 0.0).cpu().numpy().reshape(-1)[:len(X)]
        scale = np.abs(d[name]).max()
        np.testing.assert_allclose(om, d[name], rtol=0, atol=1e-12 * scale + 1e-14, err_msg=name)
    assert vm.status() == 0


def _ref_mesh_l2():
    """The level-2 mesh with the reference's (Qhull) triangle table."""
    from cmm_gpu.meshgen import icosahedral_mesh
    from cmm_gpu.mesh_functions import spherical_triangulation
    verts, _ = icosahedral_mesh(2)
    return spherical_triangulation(verts, OG.QhullLocator(verts).tris)


def test_video_driver_writes_the_reference_snapshots(sims, tmp_path):
    """euler_simulation_sphere_remapping_video: the snapshot pickles at
    steps 3, 6, 9 against the ones the reference's video driver wrote for
    the same run, and the returned submaps against its pickled stack."""
    from cmm_gpu import state_io
    mesh = _ref_mesh_l2()
    comp = sims.euler_simulation_sphere_remapping_video(8, 12, 1.0, mesh, "rossby_wave", 2 * np.pi, 5,
                                                        str(tmp_path / "run"), 3)
    for count in (3, 6, 9):
        ours = state_io.read_reference_snapshot(str(tmp_path / f"run{count}.txt"))
        ref = state_io.read_reference_snapshot(os.path.join(GOLDEN, f"ref_video_l2_run{count}.pkl"))
        assert ours["Nc"] == ref["Nc"]
        np.testing.assert_allclose(ours["vals"][:, 0], ref["vals"][:, 0], rtol=0, atol=1e-9)
    stack = np.load(str(tmp_path / "run_all_maps.npz"))
    r = state_io.reference_submaps(os.path.join(GOLDEN, "ref_video_l2_run_all_maps.pkl"))
    assert int(stack["Nc"]) == r["Nc"] == comp.Nc and list(stack["ns"]) == r["ns"]
    np.testing.assert_allclose(stack["vals"][:r["Nc"], :, 0], r["vals"][:r["Nc"], :, 0], rtol=0, atol=1e-9)


def test_reference_submap_pickle_evaluates_on_the_gpu(sims):
    """The reference's pickled composite, loaded by the restricted reader and
    assembled on the GPU, maps query points as the reference's object did."""
    from cmm_gpu import state_io
    d = np.load(os.path.join(GOLDEN, "bve_l2_L8.npz"))
    mesh, comp = state_io.composite_from_reference(os.path.join(GOLDEN, "ref_video_l2_run_all_maps.pkl"))
    img = comp(dev(d["q"])).cpu().numpy()
    np.testing.assert_allclose(img, d["img"], rtol=0, atol=1e-12)
    assert mesh.native.status() == 0


@pytest.mark.parametrize("precision", ["fp64", "split_bf16"])
def test_checkpoint_resume_is_bit_identical(sims, tmp_path, precision):
    """Stop after 7 of 22 steps, write the checkpoint, resume it in a fresh
    solver: the rest of the run is bit-identical to the uninterrupted one."""
    from cmm_gpu.meshgen import icosahedral_mesh
    verts, tris = icosahedral_mesh(3)
    args = (verts, tris, 3, 16, 24, 0.5, "rossby_wave")
    kw = dict(n_maps=5, precision=precision)
    a = sims.BVESolver(*args, **kw).run()
    b = sims.BVESolver(*args, **kw)
    b.bootstrap()
    for _ in range(7):
        b.step()
    b.save_state(str(tmp_path / "ck.npz"))
    del b
    c = sims.BVESolver(*args, **kw).load_state(str(tmp_path / "ck.npz"))
    for _ in range(24 - 2 - 7):
        c.step()
    assert (c.count, c.Nc, c.identity) == (a.count, a.Nc, a.identity)
    q = dev(np.random.default_rng(8).standard_normal((500, 3)))
    q = q / q.norm(dim=1, keepdim=True)
    assert torch.equal(a.composite(q)[0], c.composite(q)[0])
    assert torch.equal(a.omega, c.omega)
    with pytest.raises(ValueError):
        sims.BVESolver(verts, tris, 3, 16, 24, 0.5, "zonal_jet", **kw).load_state(str(tmp_path / "ck.npz"))


def test_nonfinite_initial_condition_is_reported(sims):
    """Fault injection on the host: a NaN among the initial SH coefficients
    propagates through vorticity, transform, velocity and map update without
    any out-of-range access (every location path maps NaN to a valid cell)
    and is reported as CMM_FLAG_NONFINITE; a clean run afterwards in the same
    context is unaffected."""
    from cmm_gpu import native
    from cmm_gpu.meshgen import icosahedral_mesh
    from cmm_gpu.workloads import random_sh_vorticity
    verts, tris = icosahedral_mesh(2)
    _, a = random_sh_vorticity(4, seed=1)
    bad = a.copy()
    bad[3, 4] = np.nan
    s = sims.BVESolver(verts, tris, 2, 8, 8, 1.0, sims.Vorticity(sh=bad), n_maps=3).run()
    flags = s.mesh.status(clear=True) | s.vm.status(clear=True)
    assert flags & native.FLAG_NONFINITE
    good = sims.BVESolver(verts, tris, 2, 8, 8, 1.0, sims.Vorticity(sh=a), n_maps=3).run()
    assert good.mesh.status() == 0 and good.vm.status() == 0
    assert bool(torch.isfinite(good.omega).all())


def test_reference_drivers(sims):
    """euler_simulation_sphere_remapping with the reference's signature
    against the reference's own run (bve_l2_L8.npz, its 12-step run), and
    euler_simulation_sphere (no remapping) equal to the solver's one-map run
    (to rounding: the solver evaluates its remapped map through its map
    forms, the returned sphere_diffeomorphism through its coefficient
    record)."""
    d = np.load(os.path.join(GOLDEN, "bve_l2_L8.npz"))
    mesh = _ref_mesh_l2()
    comp = sims.euler_simulation_sphere_remapping(8, 12, 1.0, mesh, "rossby_wave", rot_rate=2 * np.pi, n_maps=5)
    assert comp.Nc == int(d["Nc"]) and list(comp.ns) == list(d["ns"])
    img = comp(dev(d["q"])).cpu().numpy()
    np.testing.assert_allclose(img, d["img"], rtol=0, atol=5e-9)
    one = sims.euler_simulation_sphere(8, 12, 1.0, mesh, "rossby_wave")
    s = sims.BVESolver(mesh.vertices, mesh.simplices, 2, 8, 12, 1.0, "rossby_wave", n_maps=12).run()
    assert s.Nc == 1
    q = dev(d["q"])
    assert float((one(q).T - s.composite(q)[0]).abs().max()) < 1e-13


def test_level4_L128_whole_run_matches_reference(sims):
    """The whole barotropic configuration (level 4, L = 128, 200 steps of
    dt = 1/200, remap every 20: 10 submaps; random SH initial vorticity
    l <= 16, seed 0) against the reference driver's own run of it and the
    oracle's closed-form run (tests/golden/bve_l4_L128.npz).  Map points
    within 1e-10 and vorticity within 1e-9 relative of the closed-form run;
    within 5x the measured reference-vs-closed-form spread (the reference's
    finite-difference noise floor) of the reference's run."""
    from cmm_gpu.meshgen import icosahedral_mesh
    d = np.load(os.path.join(GOLDEN, "bve_l4_L128.npz"))
    if "img_closed" not in d:
        pytest.skip("bve_l4_L128.npz without the closed-form run")
    verts, _ = icosahedral_mesh(4)
    tris = np.load(os.path.join(GOLDEN, "mesh_l4.npz"))["tris"]
    s = sims.BVESolver(verts, tris, 4, 128, 200, 1.0, sims.Vorticity(sh=d["sh"]), n_maps=20).run()
    assert s.Nc == int(d["Nc"]) and s.ns == list(d["ns"])
    img = s.composite(dev(d["q"]))[0].cpu().numpy()
    X = img.T
    theta = np.arctan2(np.sqrt(X[0] ** 2 + X[1] ** 2), X[2])
    phi = (np.arctan2(X[1], X[0]) + 2 * np.pi) % (2 * np.pi)
    from oracle.fields import sh_series
    _, theta_q = OG.cart2sphere(d["q"].T)
    om = sh_series(d["sh"])(phi, theta) + 4 * np.pi * np.cos(theta) - 4 * np.pi * np.cos(theta_q)
    spread = np.abs(d["img_closed"] - d["img"]).max()
    e_closed = np.abs(img - d["img_closed"]).max()
    e_ref = np.abs(img - d["img"]).max()
    scale = np.abs(d["omega_closed"]).max()
    e_om = np.abs(om - d["omega_closed"]).max() / scale
    print(f"level 4 / L = 128: points vs closed-form run {e_closed:.2e}, vs reference run {e_ref:.2e} "
          f"(reference's own spread {spread:.2e}); vorticity {e_om:.2e} relative")
    assert e_closed < 1e-10
    assert e_om < 1e-9
    assert e_ref < 5 * spread + 1e-12
    assert s.mesh.status() == 0 and s.vm.status() == 0
