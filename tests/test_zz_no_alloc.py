"""The allocation-free map update, cmm_advect_project_noalloc, called
through the C ABI.

It is meant for callers that cannot allocate device memory (an application
that has given all GPU memory to its own pool, or a loop that must not call
cudaMalloc, which can synchronise the device); its scratch is a fixed array
compiled into the library.  It runs the same two kernels as the
workspace-based cmm_advect_project on the same inputs, with only the
scratch address changed, so two calls in a row must reproduce that entry
point bit for bit -- on a small mesh and on a mesh of exactly the largest
accepted size (level 5, 10242 vertices, the whole fixed array in use) --
and meshes beyond the limit must be refused.  This file is collected last
so that a run stopping at its first failure has run every other test
already; it also passes on its own in a fresh process."""
import ctypes
import os

import numpy as np
import pytest
import torch

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def nat():
    import __graft_entry__
    __graft_entry__.build()
    from cmm_gpu import native
    return native


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def call_noalloc(nat, mesh, vm, vc, ts0, scheme, t, dt, s_pts, tan, prev, jets):
    arr = (ctypes.c_void_p * len(vc))(*[c.data_ptr() for c in vc])
    return nat.lib.cmm_advect_project_noalloc(
        mesh.h, vm.h, arr, len(vc), ts0, scheme, t, dt, nat._ptr(s_pts), nat._ptr(tan),
        nat._ptr(prev), 1e-5, nat._ptr(jets), nat._stream())


def check_against_workspace_version(nat, mesh, vm, vc, s_pts, tan, cases):
    for scheme, nvs, t, pc in cases:       # calls in a row, different inputs
        ref, _ = mesh.advect_project(vm, vc[:nvs], 0.0, scheme, t, 0.1, s_pts, tan, pc)
        out = torch.full_like(ref, np.nan)
        rc = call_noalloc(nat, mesh, vm, vc[:nvs], 0.0, scheme, t, 0.1, s_pts, tan, pc, out)
        assert rc == 0, nat.lib.cmm_last_error()
        assert torch.equal(out, ref)
    assert mesh.status() == 0 and vm.status() == 0


def test_noalloc_matches_workspace_version_twice(nat):
    from cmm_gpu.meshgen import latlon_mesh_arrays, stencil_frames
    g = np.load(os.path.join(GOLDEN, "mesh_l3.npz"))
    a = np.load(os.path.join(GOLDEN, "advect_l3_L8.npz"))
    v = np.load(os.path.join(GOLDEN, "velocity_L8.npz"))
    mesh = nat.Mesh(g["verts"], g["tris"], 3)
    theta, phi, grid, verts_u = latlon_mesh_arrays(8)
    vm = nat.VelMesh(8, theta, phi, grid, verts_u)
    vc = [vm.assemble(dev(v["vals"][n])) for n in range(3)]
    tan, s_pts = stencil_frames(g["verts"])
    tan, s_pts = dev(tan), dev(s_pts)
    prev = mesh.assemble(dev(a["jets_prev"]))
    check_against_workspace_version(nat, mesh, vm, vc, s_pts, tan,
                                    [(nat.RK4, 3, 0.05, prev), (nat.EULER, 1, 0.0, None)])


def test_noalloc_at_its_size_limit(nat):
    """Level 5 has exactly the largest accepted vertex count, so the last
    scratch entries (stencil foot points of the last vertices) are used."""
    from cmm_gpu.meshgen import icosahedral_mesh, latlon_mesh_arrays, stencil_frames
    from cmm_gpu.workloads import submap_stack
    verts, tris = icosahedral_mesh(5)
    assert len(verts) == 10242
    mesh = nat.Mesh(verts, tris, 5)
    v = np.load(os.path.join(GOLDEN, "velocity_L8.npz"))
    theta, phi, grid, verts_u = latlon_mesh_arrays(8)
    vm = nat.VelMesh(8, theta, phi, grid, verts_u)
    vc = [vm.assemble(dev(v["vals"][n])) for n in range(3)]
    tan, s_pts = stencil_frames(verts)
    prev = mesh.assemble(dev(submap_stack(s_pts, tan, 1, seed=9)[0]))
    check_against_workspace_version(nat, mesh, vm, vc, dev(s_pts), dev(tan),
                                    [(nat.RK4, 3, 0.05, prev), (nat.IMPROVED_EULER, 2, 0.0, None)])


def test_noalloc_refuses_meshes_beyond_its_limit(nat):
    from cmm_gpu.meshgen import icosahedral_mesh, latlon_mesh_arrays, stencil_frames
    verts, tris = icosahedral_mesh(6)          # 40962 vertices > 10242
    mesh = nat.Mesh(verts, tris, 6)
    theta, phi, grid, verts_u = latlon_mesh_arrays(8)
    vm = nat.VelMesh(8, theta, phi, grid, verts_u)
    vc = [vm.new_coeffs()]
    tan, s_pts = stencil_frames(verts)
    jets = torch.empty((3, 4, len(verts)), dtype=torch.float64, device="cuda")
    rc = call_noalloc(nat, mesh, vm, vc, 0.0, nat.EULER, 0.0, 0.1, dev(s_pts), dev(tan), None, jets)
    assert rc == 1
    assert b"10242" in nat.lib.cmm_last_error()
