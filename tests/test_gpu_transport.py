"""GPU parity of the linear-transport path (analytic flows in the CUDA
integrators, tracer fields, the remapped transport loop) against the
reference's outputs (tests/golden/transport_l3.npz) and the oracle.

Tolerances: velocities and tracers 1e-13 absolute (CUDA's and numpy's
elementary functions differ in the last bits); foot points 1e-13.  The
remapped run against the reference: jet values 1e-10, jet gradients 3e-8,
composed points 1e-10.  Foot points of some stencils land on mesh edges,
where the reference's Qhull walk and this library's descent may pick
different neighbours; the stencil is then extrapolated in another
sub-triangle, and the gradient (a difference quotient over 4e-5) moves by
~1e-8.  The oracle replaying Qhull's choices matches the reference
bit-for-bit; the oracle with its own locator shows the same 1.1e-8 / 3.2e-11
/ 4.0e-11 as the GPU does, and the GPU is checked against that oracle run
(same tie rule) at 1e-9 / 1e-11 away from the two pole vertices, whose
stencils straddle the pole (3e-11 in their values), and at 5e-11 in the
composed points."""
import os

import numpy as np
import pytest
import torch

from conftest import GOLDEN
from oracle import evolution as EV
from oracle import transport as TR

pytestmark = pytest.mark.gpu

FLOWS = TR.FLOWS


@pytest.fixture(scope="module")
def nat():
    import __graft_entry__
    __graft_entry__.build()
    from cmm_gpu import native
    return native


@pytest.fixture(scope="module")
def gold():
    return np.load(os.path.join(GOLDEN, "transport_l3.npz"))


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def test_flow_velocities_match_reference(nat, gold):
    from cmm_gpu import dynamical_fields as F
    X = gold["X"]
    for name in FLOWS:
        U = getattr(F, name)
        for k, t in enumerate([0.0, 0.37]):
            v = U(t, 0.05, dev(X.T)).cpu().numpy()
            np.testing.assert_allclose(v, gold[f"vel_{name}_{k}"], rtol=0, atol=1e-13, err_msg=name)


def test_tracers_match_reference(nat, gold):
    from cmm_gpu import dynamical_fields as F
    X = gold["X"]
    np.testing.assert_allclose(F.static_vort_IC(0.4, dev(X.T)).cpu().numpy(), gold["tr_static_vort_IC"],
                               rtol=0, atol=1e-13)
    np.testing.assert_allclose(F.rotating_vort_IC(0.4, dev(X.T)).cpu().numpy(), gold["tr_rotating_vort_IC"],
                               rtol=0, atol=1e-13)
    mesh = F._status_mesh(torch.device("cuda", torch.cuda.current_device()))
    for kind, name in [(nat.TRACER_COSINE_BELL, "cosine_bell"), (nat.TRACER_SLOTTED_CYLINDERS, "IC_SC")]:
        got = mesh.tracer(kind, dev(X)).cpu().numpy()
        np.testing.assert_allclose(got, gold[f"tr_{name}"], rtol=0, atol=1e-12, err_msg=name)
    q = np.random.default_rng(5).standard_normal((5000, 3))
    q /= np.linalg.norm(q, axis=1)[:, None]
    np.testing.assert_allclose(F.smooth_test(dev(q)).cpu().numpy(), TR.smooth_test(q), rtol=0, atol=1e-12)
    # degree-32 series of magnitude ~10: summation order differs from scipy's
    got = F.random_initial_condition(dev(X.T)).cpu().numpy()
    np.testing.assert_allclose(got, gold["tr_random_initial_condition"], rtol=0, atol=1e-11)
    assert mesh.status(clear=True) == 0


@pytest.mark.parametrize("scheme,ofn", [(0, EV.euler_back), (1, EV.improved_euler_back), (2, EV.rk4_back),
                                        (3, EV.rk2_back)])
@pytest.mark.parametrize("name", ["u_deform_rot", "u_rotating_vortex", "u_div", "equator_vortex"])
def test_flow_integrators_match_oracle(nat, scheme, ofn, name):
    from cmm_gpu import dynamical_fields as F
    x = np.random.default_rng(9).standard_normal((3, 4000))
    x /= np.linalg.norm(x, axis=0)
    got = F._status_mesh(torch.device("cuda", 0)).flow_integrate(getattr(F, name).kind, scheme, 0.3, 0.02,
                                                                 dev(x)).cpu().numpy()
    ref = ofn(0.3, 0.02, x, TR.make_flow(name))
    np.testing.assert_allclose(got, ref, rtol=0, atol=1e-13)


def test_flow_tilted_period(nat):
    """Non-default T and alpha reach the kernels (module constants)."""
    from cmm_gpu import dynamical_fields as F
    x = np.random.default_rng(2).standard_normal((3, 300))
    x /= np.linalg.norm(x, axis=0)
    F.T, F.alpha = 2.0, 0.3
    try:
        got = F.u_deform_rot(0.7, 0.1, dev(x)).cpu().numpy()
    finally:
        F.T, F.alpha = 1, 0
    np.testing.assert_allclose(got, TR.make_flow("u_deform_rot", T=2.0, alpha=0.3)(0.7, 0.1, x),
                               rtol=0, atol=1e-13)


def test_remapped_transport_run_matches_reference(nat, gold):
    """The reference test's loop (u_deform_rot, RK4, 18 steps, remap every
    5): every remapped submap's jets and the composed images of 400 points."""
    from cmm_gpu import dynamical_fields as F
    from cmm_gpu.mesh_functions import spherical_triangulation
    from cmm_gpu.meshgen import icosahedral_mesh
    from cmm_gpu.spherical_transport import TransportSolver
    v, t = icosahedral_mesh(3)
    mesh = spherical_triangulation(v, t)
    s = TransportSolver(mesh, F.u_deform_rot, T=1.0, Nt=int(gold["Nt"]), remapping=True, n_maps=5).run()
    assert s.dt == float(gold["dt"])
    np.testing.assert_array_equal(s.jet0.cpu().numpy(), gold["jet0"])
    maps = s.maps()
    assert len(maps) == len(gold["remaps"])
    for m, ref in zip(maps, gold["remaps"]):
        got = m.vals.cpu().numpy()
        np.testing.assert_allclose(got[:, 0], ref[:, 0], rtol=0, atol=1e-10)
        np.testing.assert_allclose(got, ref, rtol=0, atol=3e-8)
    np.testing.assert_allclose(s(gold["q"]).cpu().numpy(), gold["evals"], rtol=0, atol=1e-10)
    assert mesh.native.status() == 0

    # the same loop in the oracle with this library's tie rule
    from oracle import geometry as OG
    from oracle import spline as OS
    loc = OG.ConeLocator(v, t)
    tan, s_pts = OG.stencil_points(v)
    U = TR.make_flow("u_deform_rot")
    remaps, prev, identity = [], None, True
    for count, tt in enumerate(s.tspan, start=1):
        jets = EV.advect_project(prev, EV.rk4_back, tt, s.dt, U, v, s_pts, tan, identity)
        prev, identity = OS.MapOracle(v, t, loc, jets, tie_fix=True, closed=True), False
        if count % 5 == 0:
            remaps.append(jets)
            prev, identity = None, True
    if not identity:
        remaps.append(prev.vals)
    inner = np.ones(len(v), bool)
    inner[[0, len(v) - 1]] = False   # the two pole vertices: FD stencils across the poles
    for m, ref in zip(maps, remaps):
        got = m.vals.cpu().numpy()
        np.testing.assert_allclose(got[:, 0, inner], ref[:, 0, inner], rtol=0, atol=1e-11)
        np.testing.assert_allclose(got[..., inner], ref[..., inner], rtol=0, atol=1e-9)
        np.testing.assert_allclose(got, ref, rtol=0, atol=3e-8)
    comp = OS.CompositeOracle(v, t, loc, np.stack(remaps), tie_fix=True, closed=True)
    np.testing.assert_allclose(s(gold["q"]).cpu().numpy(), comp(gold["q"]), rtol=0, atol=5e-11)


def test_reference_style_loop_equals_solver(nat):
    """advect_project_sphere(mapping, RK4_proj, t, dt, velocity.u_sbr, identity)
    written as the reference's test loop gives the solver's bits."""
    from cmm_gpu import dynamical_fields as velocity
    from cmm_gpu import evolution_functions as evol
    from cmm_gpu.mesh_functions import spherical_triangulation
    from cmm_gpu.meshgen import icosahedral_mesh, identity_jets
    from cmm_gpu.spherical_spline import sphere_diffeomorphism
    from cmm_gpu.spherical_transport import TransportSolver
    v, t = icosahedral_mesh(3)
    mesh = spherical_triangulation(v, t)
    mapping = sphere_diffeomorphism(mesh, identity_jets(v))
    tspan = np.linspace(0, 1, 12, endpoint=False)
    dt = tspan[1] - tspan[0]
    identity = True
    for tt in tspan:
        mapping = evol.advect_project_sphere(mapping, evol.RK2_proj, tt, dt, velocity.u_sbr, identity)
        identity = False
    s = TransportSolver(mesh, velocity.u_sbr, T=1.0, Nt=12, integrator=evol.RK2_proj).run()
    assert torch.equal(mapping.vals, s.mapping.vals)
    q = dev(np.random.default_rng(1).standard_normal((100, 3)))
    q = q / q.norm(dim=1, keepdim=True)
    assert torch.equal(evol.compose_maps([mapping], q), s(q))


def test_rk2_step_matches_reference(nat, gold):
    from cmm_gpu import dynamical_fields as F
    from cmm_gpu.mesh_functions import spherical_triangulation
    from cmm_gpu.meshgen import icosahedral_mesh
    v, t = icosahedral_mesh(3)
    mesh = spherical_triangulation(v, t)
    jets, _ = mesh.native.flow_advect_project(F.u_sbr.kind, nat.RK2, 0.0, 0.05, mesh.s_pts_d, mesh.tan_d, None)
    np.testing.assert_allclose(jets.cpu().numpy(), gold["jets_rk2_sbr"], rtol=0, atol=1e-10)


def test_solid_body_rotation_returns_tracer(nat):
    """Solid-body rotation over one period brings every particle back: the
    transported smooth tracer at T equals the initial one to the
    interpolation error, which falls with the mesh level."""
    from cmm_gpu import dynamical_fields as F
    from cmm_gpu.spherical_transport import TransportSolver
    q = np.random.default_rng(3).standard_normal((20000, 3))
    q /= np.linalg.norm(q, axis=1)[:, None]
    errs = [TransportSolver(level, F.u_sbr, T=1.0, Nt=2 ** level + 10).run().error(q) for level in (3, 4, 5)]
    assert errs[0] > errs[1] > errs[2], errs
    assert errs[2] < 1e-3, errs
