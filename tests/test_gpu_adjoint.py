"""GPU: the hand-written adjoints against their forward calls.

Linear maps (assembly, the SHT velocity pipeline, the SH-coefficient part of
the vorticity) by the dot-product test <A x, y> = <x, A^T y> (relative
agreement 1e-12); nonlinear ones (composition, the point part of the
vorticity) by centred differences of the forward call along random
directions (relative agreement 1e-6 at step 1e-6); the composition and the
vorticity also against torch autograd through the oracle's pure-torch FP64
restatements (normwise 1e-13)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mods():
    import __graft_entry__
    __graft_entry__.build()
    from cmm_gpu import native, adjoint, meshgen, workloads
    return native, adjoint, meshgen, workloads


def dot(a, b):
    return float((a.double() * b.double()).sum())


def test_assemble_bwd_dot_product(mods):
    native, adj, meshgen, _ = mods
    verts, tris = meshgen.icosahedral_mesh(3)
    mesh = native.Mesh(verts, tris, 3)
    g = torch.Generator(device="cuda").manual_seed(1)
    x = torch.randn((3, 4, mesh.nv), dtype=torch.float64, device="cuda", generator=g)
    y = torch.randn((mesh.nt, 64), dtype=torch.float64, device="cuda", generator=g)
    y[:, 57:] = 0
    lhs = dot(mesh.assemble(x), y)
    gj = torch.zeros_like(x)
    native.check(native.lib.cmm_assemble_bwd(mesh.h, native._ptr(y), native._ptr(gj), native._stream()), "bwd")
    rhs = dot(x, gj)
    assert abs(lhs - rhs) < 1e-12 * abs(lhs)


@pytest.mark.parametrize("L", [8, 17, 32])
def test_sht_velocity_bwd_dot_product(mods, L):
    native, adj, meshgen, _ = mods
    theta, phi, grid, verts = meshgen.latlon_mesh_arrays(L)
    vm = native.VelMesh(L, theta, phi, grid, verts)
    sht = native.Sht(L)
    g = torch.Generator(device="cuda").manual_seed(L)
    om = torch.randn((L + 1, 2 * L), dtype=torch.float64, device="cuda", generator=g)
    ybar = torch.randn((3, 4, vm.nv), dtype=torch.float64, device="cuda", generator=g)
    lhs = dot(sht.velocity(vm, om), ybar)
    gw = torch.empty_like(om)
    native.check(native.lib.cmm_sht_velocity_bwd(sht.h, vm.h, native._ptr(ybar), native._ptr(gw),
                                                 native._stream()), "bwd")
    rhs = dot(om, gw)
    print(f"L={L}: <V w, y> = {lhs:.15e}, <w, V^T y> = {rhs:.15e}")
    assert abs(lhs - rhs) < 1e-11 * (abs(lhs) + abs(rhs))


def test_compose_bwd_against_differences(mods):
    native, adj, meshgen, workloads = mods
    verts, tris = meshgen.icosahedral_mesh(3)
    mesh = native.Mesh(verts, tris, 3)
    tan, s_pts = meshgen.stencil_frames(verts)
    jets = workloads.submap_stack(s_pts, tan, 3, seed=2)
    cs = [mesh.assemble(torch.from_numpy(j).cuda()) for j in jets]
    q = torch.from_numpy(meshgen.random_sphere_points(3000, seed=4)).cuda()
    g = torch.Generator(device="cuda").manual_seed(5)
    y = torch.randn_like(q)
    cs_v = [c.clone().requires_grad_(True) for c in cs]
    qv = q.clone().requires_grad_(True)
    out = adj.Compose.apply(qv, mesh, *cs_v)
    (out * y).sum().backward()
    h = 1e-6
    for k in range(3):   # direction in submap k's used ordinates
        d = torch.randn(cs[k].shape, dtype=torch.float64, device="cuda", generator=g)
        d[:, 57:] = 0
        def J(sgn):
            cc = [c.clone() for c in cs]
            cc[k] = cc[k] + sgn * h * d
            return dot(mesh.compose(cc, q)[0], y)
        fd = (J(1) - J(-1)) / (2 * h)
        ad = dot(cs_v[k].grad, d)
        assert abs(fd - ad) < 1e-6 * abs(ad), (k, fd, ad)
    dq = torch.randn(q.shape, dtype=torch.float64, device="cuda", generator=g)
    dq -= (dq * q).sum(1, keepdim=True) * q
    fd = (dot(mesh.compose(cs, q + h * dq)[0], y) - dot(mesh.compose(cs, q - h * dq)[0], y)) / (2 * h)
    assert abs(fd - dot(qv.grad, dq)) < 1e-6 * abs(fd)


def test_compose_bwd_matches_autograd_restatement(mods):
    """The composition's hand-written backward (cmm_compose_bwd) against a
    reference FP64 gradient: torch autograd on the CPU through the pure-torch
    restatement of the oracle's composition (oracle/compose_torch.py, pinned
    to the numpy oracle by tests/test_oracle_autograd.py), with the same
    triangle and sub-triangle choices held fixed.  Gradients with respect to
    the ordinates of each of 3 submaps (level 3) and to 3000 query points
    agree normwise to 1e-13 (measured 4e-15..8e-15)."""
    from oracle import geometry as G
    from oracle.compose_torch import composite_eval
    native, adj, meshgen, workloads = mods
    verts, tris = meshgen.icosahedral_mesh(3)
    nt = len(tris)
    mesh = native.Mesh(verts, tris, 3)
    tan, s_pts = meshgen.stencil_frames(verts)
    jets = workloads.submap_stack(s_pts, tan, 3, seed=2)
    cs = [mesh.assemble(torch.from_numpy(j).cuda()) for j in jets]
    q = torch.from_numpy(meshgen.random_sphere_points(3000, seed=4)).cuda()
    y = torch.randn(q.shape, dtype=torch.float64, generator=torch.Generator().manual_seed(6))
    cs_v = [c.clone().requires_grad_(True) for c in cs]
    qv = q.clone().requires_grad_(True)
    (adj.Compose.apply(qv, mesh, *cs_v) * y.cuda()).sum().backward()
    # the same ordinates in the reference layout (3,19,Nt), on the CPU
    ref = [c.detach().cpu()[:, :57].reshape(nt, 19, 3).permute(2, 1, 0).contiguous().requires_grad_(True)
           for c in cs]
    qr = q.cpu().clone().requires_grad_(True)
    (composite_eval(ref, qr, verts, tris, G.ConeLocator(verts, tris)) * y).sum().backward()

    def rel(a, b):
        return float((a - b).norm() / b.norm())
    for k in range(3):
        g_gpu = cs_v[k].grad.cpu()
        e = rel(g_gpu[:, :57].reshape(nt, 19, 3).permute(2, 1, 0), ref[k].grad)
        print(f"submap {k}: ordinate gradient rel err {e:.2e}")
        assert e < 1e-13
    e = rel(qv.grad.cpu(), qr.grad)
    print(f"query-point gradient rel err {e:.2e}")
    assert e < 1e-13


def test_vorticity_bwd(mods):
    native, adj, meshgen, workloads = mods
    L = 16
    theta, phi, grid, verts = meshgen.latlon_mesh_arrays(L)
    vm = native.VelMesh(L, theta, phi, grid, verts)
    _, a = workloads.random_sh_vorticity(6, seed=1)
    sh = torch.from_numpy(a).cuda()
    X = torch.from_numpy(meshgen.random_sphere_points((L + 1) * 2 * L, seed=2)).cuda()
    g = torch.Generator(device="cuda").manual_seed(3)
    y = torch.randn((L + 1, 2 * L), dtype=torch.float64, device="cuda", generator=g)
    rot = 2 * np.pi
    Xv, shv = X.clone().requires_grad_(True), sh.clone().requires_grad_(True)
    (adj.Vorticity.apply(Xv, shv, vm, rot) * y).sum().backward()
    # SH coefficients: linear
    d = torch.randn(sh.shape, dtype=torch.float64, device="cuda", generator=g)
    for l in range(sh.shape[0]):
        d[l, 2 * l + 1:] = 0
    w1 = vm.vorticity(native.VORT_NONE, [], X, rot, sh=sh + d)
    w0 = vm.vorticity(native.VORT_NONE, [], X, rot, sh=sh)
    assert abs(dot(w1 - w0, y) - dot(shv.grad, d)) < 1e-11 * abs(dot(shv.grad, d))
    # points: tangent directions, centred differences on the sphere
    dX = torch.randn(X.shape, dtype=torch.float64, device="cuda", generator=g)
    dX -= (dX * X).sum(1, keepdim=True) * X
    h = 1e-6
    wp = vm.vorticity(native.VORT_NONE, [], X + h * dX, rot, sh=sh)
    wm = vm.vorticity(native.VORT_NONE, [], X - h * dX, rot, sh=sh)
    fd = dot(wp - wm, y) / (2 * h)
    assert abs(fd - dot(Xv.grad, dX)) < 1e-6 * abs(fd)


def test_vorticity_bwd_matches_autograd_restatement(mods):
    """The vorticity's hand-written backward (cmm_vorticity_bwd) against
    torch autograd on the CPU through the oracle's pure-torch restatement of
    the SH series and the planetary term (oracle/vorticity_torch.py, pinned
    to oracle.fields.sh_series by tests/test_oracle_autograd.py): the
    coefficient gradient on the used entries (|m| <= l) and the tangent part
    of the point gradient, L = 16, l <= 6, normwise to 1e-13 (measured
    9e-16 and 1.4e-16)."""
    from oracle.vorticity_torch import sampled_vorticity
    native, adj, meshgen, workloads = mods
    L = 16
    theta, phi, grid, verts = meshgen.latlon_mesh_arrays(L)
    vm = native.VelMesh(L, theta, phi, grid, verts)
    _, a = workloads.random_sh_vorticity(6, seed=1)
    X = torch.from_numpy(meshgen.random_sphere_points((L + 1) * 2 * L, seed=2))
    y = torch.randn((L + 1, 2 * L), dtype=torch.float64, generator=torch.Generator().manual_seed(3))
    rot = 2 * np.pi
    Xv, shv = X.cuda().requires_grad_(True), torch.from_numpy(a).cuda().requires_grad_(True)
    (adj.Vorticity.apply(Xv, shv, vm, rot) * y.cuda()).sum().backward()
    Xr, shr = X.clone().requires_grad_(True), torch.from_numpy(a.copy()).requires_grad_(True)
    (sampled_vorticity(shr, Xr, rot, 0.0) * y.reshape(-1)).sum().backward()

    def rel(u, v):
        return float((u - v).norm() / v.norm())
    used = torch.zeros(shr.shape, dtype=torch.bool)
    for l in range(used.shape[0]):
        used[l, :2 * l + 1] = True
    e = rel(shv.grad.cpu()[used], shr.grad[used])
    print(f"coefficient gradient rel err {e:.2e}")
    assert e < 1e-13

    def tangent(g):
        return g - (g * X).sum(1, keepdim=True) * X
    e = rel(tangent(Xv.grad.cpu()), tangent(Xr.grad))
    print(f"point gradient (tangent) rel err {e:.2e}")
    assert e < 1e-13


@pytest.mark.parametrize("scheme,nvs,with_prev", [(0, 1, False), (1, 2, False), (2, 2, True), (2, 3, True),
                                                  (2, 3, False)])
def test_advect_bwd_against_differences(mods, scheme, nvs, with_prev):
    """cmm_advect_project_bwd along random directions in the velocity
    records and the previous map's records (centred differences, step 1e-6)."""
    native, adj, meshgen, workloads = mods
    L, level = 16, 3
    verts, tris = meshgen.icosahedral_mesh(level)
    mesh = native.Mesh(verts, tris, level)
    theta, phi, grid, vverts = meshgen.latlon_mesh_arrays(L)
    vm = native.VelMesh(L, theta, phi, grid, vverts)
    sht = native.Sht(L)
    Th, Ph = np.meshgrid(theta, phi, indexing="ij")
    vel = []
    for k in range(3):
        om = 30 * np.cos(Th) * np.cos(4 * Ph + k) * np.sin(Th) ** 4 + 3 * np.sin(2 * Ph) * np.sin(Th) ** 2
        vel.append(vm.assemble(sht.velocity(vm, torch.from_numpy(om).cuda())))
    tan, s_pts = meshgen.stencil_frames(verts)
    tan, s_pts = torch.from_numpy(np.ascontiguousarray(tan)).cuda(), torch.from_numpy(np.ascontiguousarray(s_pts)).cuda()
    jets0 = workloads.submap_stack(meshgen.stencil_frames(verts)[1], meshgen.stencil_frames(verts)[0], 1, seed=8)[0]
    prev = mesh.assemble(torch.from_numpy(jets0).cuda()) if with_prev else torch.empty(0, dtype=torch.float64, device="cuda")
    ts0, t, dt = 0.0, 0.02, 0.01
    g = torch.Generator(device="cuda").manual_seed(11)
    y = torch.randn((3, 4, mesh.nv), dtype=torch.float64, device="cuda", generator=g)
    # the two pole vertices' stencils straddle the lat-lon mesh's polar fans,
    # where their foot points are not smooth enough for centred differences
    # at this step (the adjoint's piecewise derivative is still exact there)
    y[:, :, 0] = 0
    y[:, :, -1] = 0
    vv = [v.clone().requires_grad_(True) for v in vel]
    pv = prev.clone().requires_grad_(with_prev)
    args = (mesh, vm, nvs, ts0, scheme, t, dt, s_pts, tan)
    jets = adj.AdvectProject.apply(pv, vv[0], vv[1], vv[2], *args)
    (jets * y).sum().backward()
    h = 1e-6

    def J(vel_, prev_):
        out, _ = mesh.advect_project(vm, vel_[:nvs], ts0, scheme, t, dt, s_pts, tan,
                                     prev_ if with_prev else None)
        return dot(out, y)

    for k in range(nvs):
        d = torch.randn(vel[k].shape, dtype=torch.float64, device="cuda", generator=g) * vel[k].abs().max()
        d[:, 57:] = 0
        vp = [v.clone() for v in vel]
        vm_ = [v.clone() for v in vel]
        vp[k] += h * d
        vm_[k] -= h * d
        fd = (J(vp, prev) - J(vm_, prev)) / (2 * h)
        ad = dot(vv[k].grad, d)
        print(f"scheme {scheme} nvs {nvs} level {k}: fd {fd:.10e} adjoint {ad:.10e}")
        assert abs(fd - ad) < 1e-6 * abs(ad) + 1e-9
    if with_prev:
        d = torch.randn(prev.shape, dtype=torch.float64, device="cuda", generator=g)
        d[:, 57:] = 0
        fd = (J(vel, prev + h * d) - J(vel, prev - h * d)) / (2 * h)
        ad = dot(pv.grad, d)
        print(f"prev: fd {fd:.10e} adjoint {ad:.10e}")
        assert abs(fd - ad) < 1e-6 * abs(ad)


def test_bve_gradient_against_differences(mods):
    """dJ/d(initial SH coefficients) of a whole small run (level 3, L=16,
    14 steps, remap every 5, checkpointed) against centred differences of
    J on 8 random coefficients.  The differences of J carry the map
    update's amplified rounding (stencil differences over 4e-5 turn 1e-16
    into ~3e-12 per jet gradient, every step) and, at large steps, the
    curvature of J: their own error is ~1e-7..1e-5 depending on the step.
    The check takes the best of steps 1e-4, 1e-5, 1e-6 and requires the
    discrepancy below 2e-6 of the coefficient's derivative or, for the
    small derivatives where the differences' own noise dominates, below
    1e-7 of the largest derivative."""
    native, adj, meshgen, workloads = mods
    lmax = 6
    run = adj.BVEGradient(3, 16, 14, 0.1, n_maps=5)
    _, a = workloads.random_sh_vorticity(lmax, seed=1)
    _, b = workloads.random_sh_vorticity(lmax, seed=2)
    sh = torch.from_numpy(a).cuda()
    with torch.no_grad():
        target = run.omega_T(sh + 0.1 * torch.from_numpy(b).cuda())
    J, grad = run.gradient(sh, target)
    rng = np.random.default_rng(5)
    idx = [(l, int(rng.integers(0, 2 * l + 1))) for l in rng.integers(1, lmax + 1, 8)]
    gmax = float(grad.abs().max())
    for l, c in idx:
        ad = float(grad[l, c])
        errs = []
        for h in (1e-4, 1e-5, 1e-6):
            sp, sm = sh.clone(), sh.clone()
            sp[l, c] += h
            sm[l, c] -= h
            with torch.no_grad():
                fd = (float(run.misfit(sp, target)) - float(run.misfit(sm, target))) / (2 * h)
            errs.append(abs(fd - ad))
        print(f"coefficient ({l},{c - l}): adjoint {ad:.10e} rel err at h=1e-4,1e-5,1e-6: "
              + " ".join(f"{e / abs(ad):.1e}" for e in errs))
        assert min(errs) < max(2e-6 * abs(ad), 1e-7 * gmax)


def test_bve_gradient_matches_whole_run_restatement(mods):
    """dJ/d(initial SH coefficients) of a whole small run (level 3, L = 8,
    10 steps, remap every 4: bootstrap, remaps, velocity-level rotation)
    against the reference FP64 gradient of a pure-torch restatement of the
    whole run on the CPU (oracle.bve_torch, torch autograd through every
    stage with the same piecewise choices), every coefficient.  The two
    forward runs agree to the map update's rounding floor (stencil
    differences over 4e-5 amplify rounding 2.5e4 times per step, ~1e-11);
    asserted: omega_T within 1e-10 and the gradient within 1e-8 normwise and
    1e-8 of its largest entry per coefficient."""
    native, adj, meshgen, workloads = mods
    from oracle.bve_torch import BVETorch
    verts, tris = meshgen.icosahedral_mesh(3)
    run = adj.BVEGradient(3, 8, 10, 0.05, n_maps=4)
    _, a = workloads.random_sh_vorticity(6, seed=1)
    _, b = workloads.random_sh_vorticity(6, seed=2)
    sh = torch.from_numpy(a).cuda()
    with torch.no_grad():
        target = run.omega_T(sh + 0.1 * torch.from_numpy(b).cuda())
        om = run.omega_T(sh).cpu().numpy()
    J, grad = run.gradient(sh, target)
    grad = grad.cpu().numpy()
    bt = BVETorch(verts, tris, 8, 10, 0.05, n_maps=4)
    om_t = bt.omega_T(torch.from_numpy(a)).detach().numpy()
    Jt, gt = bt.gradient(a, target.cpu().numpy())
    e_om = np.abs(om - om_t).max() / np.abs(om_t).max()
    e_norm = np.linalg.norm(grad - gt) / np.linalg.norm(gt)
    e_max = np.abs(grad - gt).max() / np.abs(gt).max()
    print(f"whole run vs torch restatement: omega_T {e_om:.2e}, J {abs(J - Jt) / Jt:.2e}, "
          f"gradient normwise {e_norm:.2e}, per coefficient {e_max:.2e} of the largest")
    assert e_om < 1e-10
    assert abs(J - Jt) < 1e-9 * Jt
    assert e_norm < 1e-8 and e_max < 1e-8
