"""GPU parity: lat-lon velocity mesh location, the velocity interpolant, the
backward integrators and the CMM map update against the reference's golden
outputs and the oracle.

Tolerances: lat-lon triangle ids bit-exact; velocities within 1e-12
(relative to max |u|); foot points within 1e-13; new jet values within
1e-12; jet gradients (centred differences with step 1e-5, which amplify
rounding by 1e5) within 1e-9."""
import os

import numpy as np
import pytest
import torch

from conftest import GOLDEN
from oracle import geometry as OG
from oracle import spline as OS
from oracle import evolution as OE

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def nat():
    import __graft_entry__
    __graft_entry__.build()
    from cmm_gpu import native
    return native


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    return t.cpu().numpy()


def golden(name):
    return np.load(os.path.join(GOLDEN, name))


def velmesh(nat, L):
    from cmm_gpu.meshgen import latlon_mesh_arrays
    theta, phi, grid, verts = latlon_mesh_arrays(L)
    return nat.VelMesh(L, theta, phi, grid, verts), verts


def test_latlon_arrays_match_reference():
    from cmm_gpu.meshgen import latlon_mesh_arrays
    d = golden("velocity_L8.npz")
    theta, phi, grid, verts = latlon_mesh_arrays(8)
    np.testing.assert_array_equal(verts, d["verts"])


def test_latlon_locate_matches_reference(nat):
    """Bit-exact triangle ids, except queries lying on a triangle edge or
    vertex (ring points, meridians), which may resolve to another triangle
    that contains them."""
    d = golden("velocity_L8.npz")
    vm, verts = velmesh(nat, 8)
    tri, bcc = vm.locate(dev(d["q"]))
    tri, bcc = host(tri), host(bcc)
    mu = OG.LatLonMesh(8)
    diff = tri != d["tri"]
    on_edge = OG.edge_distance(mu.vertices, mu.simplices, d["tri"], d["q"]) <= 1e-14
    assert not (diff & ~on_edge).any(), np.nonzero(diff & ~on_edge)
    assert (bcc[diff].min(axis=1) >= -1e-13).all()
    same = ~diff
    np.testing.assert_allclose(bcc[same], d["bcc"][same], rtol=0, atol=1e-13)
    print(f"{diff.sum()} of {len(tri)} edge/vertex queries resolved to another container")


@pytest.mark.parametrize("L", [16, 128, 1024])
def test_latlon_locate_random(nat, L):
    from cmm_gpu.meshgen import random_sphere_points
    q = random_sphere_points(100_000, seed=L)
    vm, _ = velmesh(nat, L)
    tri, _ = vm.locate(dev(q))
    _, ref, _ = OG.LatLonMesh(L).query(q)
    np.testing.assert_array_equal(host(tri), ref)


def vel_coeffs(nat, vm, vals):
    return [vm.assemble(dev(vals[n])) for n in range(3)]


def test_velocity_matches_reference(nat):
    d = golden("velocity_L8.npz")
    vm, _ = velmesh(nat, 8)
    vc = vel_coeffs(nat, vm, d["vals"])
    rec = host(vc[1])[:, :57].reshape(-1, 19, 3).transpose(2, 1, 0)
    np.testing.assert_allclose(rec, d["coeffs"][1], rtol=0, atol=1e-12)
    u = host(vm.velocity(vc, 0.0, float(d["t"]), float(d["dt"]), dev(d["q"].T)))
    scale = np.abs(d["vel"]).max()
    np.testing.assert_allclose(u / scale, d["vel"] / scale, rtol=0, atol=1e-12)
    for nvs in (1, 2):
        u = host(vm.velocity(vc[:nvs], 0.0, 0.17, 0.1, dev(d["q"].T)))
        U = OS.VelocityOracle(OG.LatLonMesh(8), d["vals"], d["ts"])
        for n in range(3):
            U.init_coeffs(n)
        U.nVs = nvs
        np.testing.assert_allclose(u / scale, U(0.17, 0.1, d["q"].T) / scale, rtol=0, atol=1e-12)


@pytest.mark.parametrize("scheme,nvs", [(0, 1), (1, 2), (2, 3)])
def test_integrators_against_oracle(nat, scheme, nvs):
    from cmm_gpu.meshgen import random_sphere_points
    d = golden("velocity_L8.npz")
    vm, _ = velmesh(nat, 8)
    vc = vel_coeffs(nat, vm, d["vals"])[:nvs]
    x = random_sphere_points(5000, seed=scheme).T.copy()
    out = host(vm.integrate(vc, 0.0, scheme, 0.05, 0.1, dev(x)))
    U = OS.VelocityOracle(OG.LatLonMesh(8), d["vals"], d["ts"])
    for n in range(3):
        U.init_coeffs(n)
    U.nVs = nvs
    f = [OE.euler_back, OE.improved_euler_back, OE.rk4_back][scheme]
    ref = f(0.05, 0.1, x, U)
    np.testing.assert_allclose(out, ref, rtol=0, atol=1e-13)


def test_advect_project_matches_reference(nat):
    a, m, v = golden("advect_l3_L8.npz"), golden("mesh_l3.npz"), golden("velocity_L8.npz")
    verts, tris = m["verts"], m["tris"]
    mesh = nat.Mesh(verts, tris, 3)
    vm, _ = velmesh(nat, 8)
    vc = vel_coeffs(nat, vm, v["vals"])
    tan, s_pts = OG.stencil_points(verts)
    prev = mesh.assemble(dev(a["jets_prev"]))
    jets, work = mesh.advect_project(vm, vc, 0.0, nat.RK4, 0.05, 0.1, dev(s_pts), dev(tan), prev)
    jets, yn = host(jets), host(work)[:3 * len(verts)].reshape(3, -1)
    # the reference integrates the same points (RK4_proj) -> foot points
    U = OS.VelocityOracle(OG.LatLonMesh(8), v["vals"], v["ts"])
    for n in range(3):
        U.init_coeffs(n)
    U.nVs = 3
    yref = OE.rk4_back(0.05, 0.1, verts.T, U)
    np.testing.assert_allclose(yn, yref, rtol=0, atol=1e-13)
    # vertices whose foot point lies on a mesh edge may be evaluated in
    # either neighbouring triangle (the reference's Qhull choice is one)
    loc = OG.QhullLocator(verts)
    near = OG.edge_distance(verts, tris, loc.locate(yref.T), yref.T) <= 1e-14
    ok = ~near
    # (1) against the oracle evaluated in closed form (the same linear maps
    #     with the per-triangle inverse vertex matrix the kernels use)
    prev_o = OS.MapOracle(verts, tris, loc, a["jets_prev"], closed=True)
    sn = OE.rk4_back(0.05, 0.1, s_pts.reshape(3, -1), U).reshape(s_pts.shape)
    jo = OE.jets_from_stencil(prev_o.stencil_eval(yref, sn), tan)
    np.testing.assert_allclose(jets[:, 0][:, ok], jo[:, 0][:, ok], rtol=0, atol=1e-12)
    # rounding differences (~1e-15: FMA contraction, summation order) times
    # the 1/(4 eps) = 2.5e4 difference quotient
    np.testing.assert_allclose(jets[:, 1:][..., ok], jo[:, 1:][..., ok], rtol=0, atol=5e-10)
    # (2) against the reference: values within 1e-12; gradients within the
    #     reference's own rounding noise (its four per-point determinant
    #     evaluations round independently and the 1/(4 eps) difference
    #     amplifies that by 2.5e4: the closed-form oracle differs from the
    #     reference by up to ~9e-9 here)
    ref = a["jets_rk4"]
    noise = np.abs(jo[:, 1:][..., ok] - ref[:, 1:][..., ok]).max()
    assert noise < 2e-8
    np.testing.assert_allclose(jets[:, 0][:, ok], ref[:, 0][:, ok], rtol=0, atol=1e-12)
    np.testing.assert_allclose(jets[:, 1:][..., ok], ref[:, 1:][..., ok], rtol=0, atol=2 * noise + 1e-10)
    np.testing.assert_allclose(jets[..., near], ref[..., near], rtol=0, atol=1e-6)
    for scheme, nvs, key in ((nat.EULER, 1, "jets_euler"), (nat.IMPROVED_EULER, 2, "jets_ieuler")):
        j, _ = mesh.advect_project(vm, vc[:nvs], 0.0, scheme, 0.0, 0.1, dev(s_pts), dev(tan), None)
        j = host(j)
        np.testing.assert_allclose(j[:, 0], a[key][:, 0], rtol=0, atol=1e-12)
        np.testing.assert_allclose(j[:, 1:], a[key][:, 1:], rtol=0, atol=1e-9)
    assert mesh.status() == 0 and vm.status() == 0


def test_fp32_velocity_records(nat):
    """cmm_velmesh_set_records(CMM_REC_FP32): FP32 ordinates and FP32
    patches against the FP64 records on the same velocity jets; stated
    error 1e-6 of max |u| (FP32 rounding of ordinates ~1e-7 relative), and
    the RK4 foot points (FP64 accumulation) within dt * 1e-6 * max |u|."""
    from cmm_gpu.meshgen import random_sphere_points
    d = golden("velocity_L8.npz")
    vm64, _ = velmesh(nat, 8)
    vm32, _ = velmesh(nat, 8)
    vm32.set_records(nat.VelMesh.REC_FP32)
    c64 = vel_coeffs(nat, vm64, d["vals"])
    c32 = vel_coeffs(nat, vm32, d["vals"])
    assert c32[0].dtype == torch.float32
    np.testing.assert_allclose(host(c32[1]), host(c64[1]).astype(np.float32), rtol=2e-6, atol=1e-6)
    x = random_sphere_points(20000, seed=11).T.copy()
    u64 = host(vm64.velocity(c64, 0.0, 0.13, 0.1, dev(x)))
    u32 = host(vm32.velocity(c32, 0.0, 0.13, 0.1, dev(x)))
    scale = np.abs(u64).max()
    err = np.abs(u32 - u64).max() / scale
    print(f"FP32 velocity records: relative velocity error {err:.2e}")
    assert 1e-10 < err < 1e-6
    f64 = host(vm64.integrate(c64, 0.0, 2, 0.05, 0.1, dev(x)))
    f32 = host(vm32.integrate(c32, 0.0, 2, 0.05, 0.1, dev(x)))
    assert np.abs(f32 - f64).max() < 0.1 * 1e-6 * scale
