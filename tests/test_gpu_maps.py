"""GPU parity: point location, assembly, map evaluation, composition,
stencil evaluation and Jacobians of libcmmgpu.so against the oracle and the
reference's golden outputs.

Tolerances: triangle ids bit-exact except for queries within 1e-14 of an
edge of the oracle's triangle (either neighbour contains them; counted);
FP64 map coordinates within 1e-12 (relative to |X| = 1); barycentrics and
ordinates within 1e-13; Jacobians within 1e-10 (relative to |J|)."""
import os

import numpy as np
import pytest
import torch

from conftest import GOLDEN
from oracle import geometry as OG
from oracle import spline as OS

pytestmark = pytest.mark.gpu
EDGE_TOL = 1e-14


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


def coeff_record_to_ref(rec, nt):
    """(nt,64) device record -> reference layout (3,19,nt)."""
    return rec[:, :57].reshape(nt, 19, 3).transpose(2, 1, 0)


@pytest.mark.parametrize("level", [3, 4])
def test_locate_matches_reference_qhull(nat, level):
    d = golden(f"mesh_l{level}.npz")
    m = nat.Mesh(d["verts"], d["tris"], level)
    tri, bcc = m.locate(dev(d["q"]))
    tri, bcc = host(tri), host(bcc)
    diff = tri != d["tri"]
    near = OG.edge_distance(d["verts"], d["tris"], d["tri"], d["q"]) <= EDGE_TOL
    assert not (diff & ~near).any()
    # a disagreement is another container of the query
    assert (OG.edge_distance(d["verts"], d["tris"], tri[diff], d["q"][diff]) <= EDGE_TOL).all()
    same = ~diff
    np.testing.assert_allclose(bcc[same], d["bcc"][same], rtol=0, atol=1e-13)
    assert m.status() == 0
    print(f"level {level}: {diff.sum()} of {len(tri)} near-edge queries resolved to the neighbour")


def qhull_case(level):
    """The Qhull-order fixture of a large level (tests/golden/make_golden.py
    qhull_fixture): the reference's triangle table and find_simplex ids of
    seeded random queries; vertices and queries regenerated here and
    checked against the fixture's digests."""
    import hashlib
    from cmm_gpu.meshgen import icosahedral_mesh, random_sphere_points
    d = golden(f"qhull_l{level}.npz")
    verts, _ = icosahedral_mesh(level)
    assert hashlib.sha256(np.ascontiguousarray(verts).tobytes()).hexdigest() == str(d["verts_sha"])
    qr = random_sphere_points(int(d["nq"]), seed=int(d["seed"]))
    assert hashlib.sha256(np.ascontiguousarray(qr).tobytes()).hexdigest() == str(d["q_sha"])
    return verts, d["tris"], np.concatenate([qr, d["q_special"]]), d["tri"], d["bcc"]


@pytest.mark.parametrize("level", [5, 6])
def test_locate_matches_reference_qhull_large_levels(nat, level):
    """Bit-exact triangle ids in the reference's own (Qhull) row order at
    levels 5 and 6, except within 1e-14 of an edge (counted)."""
    if not os.path.exists(os.path.join(GOLDEN, f"qhull_l{level}.npz")):
        pytest.skip(f"qhull_l{level}.npz not generated")
    verts, tris, q, ref_tri, ref_bcc = qhull_case(level)
    m = nat.Mesh(verts, tris, level)
    tri, bcc = m.locate(dev(q))
    tri, bcc = host(tri), host(bcc)
    diff = tri != ref_tri
    near = OG.edge_distance(verts, tris, ref_tri, q) <= EDGE_TOL
    assert not (diff & ~near).any(), int((diff & ~near).sum())
    assert (OG.edge_distance(verts, tris, tri[diff], q[diff]) <= EDGE_TOL).all()
    # barycentrics: the reference's determinant ratios carry a rounding
    # error ~eps/h^2 (h the edge length), which grows 4x per level: 1e-13
    # at level 4, scaled by 4 per level above it
    same = ~diff
    np.testing.assert_allclose(bcc[same], ref_bcc[same], rtol=0, atol=1e-13 * 4.0 ** (level - 4))
    assert m.status() == 0
    print(f"level {level}: {int(near.sum())} queries within 1e-14 of an edge, "
          f"{int(diff.sum())} resolved to the neighbour, of {len(tri)}")


@pytest.mark.parametrize("level", [5, 7])
def test_locate_large_levels_against_cone_oracle(nat, level):
    from cmm_gpu.meshgen import icosahedral_mesh, random_sphere_points
    verts, tris = icosahedral_mesh(level)
    q = random_sphere_points(200_000, seed=level)
    m = nat.Mesh(verts, tris, level)
    tri, bcc = m.locate(dev(q))
    tri = host(tri)
    ref = OG.ConeLocator(verts, tris).locate(q)
    diff = tri != ref
    near = OG.edge_distance(verts, tris, ref, q) <= EDGE_TOL
    assert not (diff & ~near).any()
    b = host(bcc)
    assert b.min() > -1e-12
    assert m.status() == 0


def test_assemble_matches_reference(nat):
    d, g = golden("map_l3.npz"), golden("mesh_l3.npz")
    m = nat.Mesh(g["verts"], g["tris"], 3)
    rec = host(m.assemble(dev(d["jets"][0])))
    np.testing.assert_allclose(coeff_record_to_ref(rec, len(g["tris"])), d["coeffs0"], rtol=0, atol=1e-13)


def test_map_eval_and_composite_match_reference(nat):
    d, g = golden("map_l3.npz"), golden("mesh_l3.npz")
    m = nat.Mesh(g["verts"], g["tris"], 3)
    cs = [m.assemble(dev(j)) for j in d["jets"]]
    out, tri, _, _ = m.compose(cs[:1], dev(d["q"]), want_tri=True)
    out = host(out)
    # split-centre ties: the reference's three barycentrics are bitwise
    # equal, its tables select the degenerate sub-triangle (v1,v1,v1) and it
    # returns NaN or, when the 0/0 determinants round to finite values, the
    # vertex ordinate c0.  The spline's value there is the centre ordinate,
    # which the library returns (equal to the tie-broken oracle).
    b = g["bcc"]
    tie = (b[:, 0] == b[:, 1]) & (b[:, 1] == b[:, 2])
    assert tie.sum() > 0 and (~np.isfinite(d["img"]).all(0) <= tie).all()
    ok = ~tie
    np.testing.assert_allclose(out[ok], d["img"].T[ok], rtol=0, atol=1e-12)
    orc = OS.MapOracle(g["verts"], g["tris"], OG.ConeLocator(g["verts"], g["tris"]), d["jets"][0],
                       tie_fix=True)
    np.testing.assert_allclose(out[tie], orc(d["q"][tie]).T, rtol=0, atol=1e-12)
    cout, _, _, _ = m.compose(cs, dev(d["q"]))
    cout = host(cout)
    fin = np.isfinite(d["comp_img"]).all(1) & ~tie
    np.testing.assert_allclose(cout[fin], d["comp_img"][fin], rtol=0, atol=1e-12)
    assert np.isfinite(cout).all()
    assert m.status() == 0


def test_stencil_eval_matches_reference(nat):
    d, g = golden("map_l3.npz"), golden("mesh_l3.npz")
    m = nat.Mesh(g["verts"], g["tris"], 3)
    c = m.assemble(dev(d["jets"][0]))
    st = host(m.stencil_eval(c, dev(d["yn"]), dev(d["sp"])))
    np.testing.assert_allclose(st, d["st"], rtol=0, atol=1e-12)


def make_stack(level, S, seed):
    from cmm_gpu.meshgen import icosahedral_mesh
    from cmm_gpu.workloads import submap_stack
    verts, tris = icosahedral_mesh(level)
    tan, s_pts = OG.stencil_points(verts)
    return verts, tris, submap_stack(s_pts, tan, S, seed=seed)


def test_composition_level5_eight_submaps(nat):
    from cmm_gpu.meshgen import random_sphere_points
    verts, tris, jets = make_stack(5, 8, seed=11)
    q = random_sphere_points(20_000, seed=12)
    m = nat.Mesh(verts, tris, 5)
    cs = [m.assemble(dev(j)) for j in jets]
    out, tri, tri_all, _ = m.compose(cs, dev(q), want_tri=True, want_tri_all=True)
    comp = OS.CompositeOracle(verts, tris, OG.ConeLocator(verts, tris), jets, tie_fix=True)
    ref, rtri, pts = comp(q, record=True)
    np.testing.assert_allclose(host(out), ref, rtol=0, atol=1e-12)
    ta = host(tri_all)[::-1]          # application order: submap S-1 first
    np.testing.assert_array_equal(host(tri), ta[0])
    for s in range(8):
        diff = ta[s] != rtri[s]
        near = OG.edge_distance(verts, tris, rtri[s], pts[s]) <= 1e-13
        assert not (diff & ~near).any(), s


def test_jacobian_against_oracle_and_differences(nat):
    from cmm_gpu.meshgen import random_sphere_points
    verts, tris, jets = make_stack(4, 3, seed=21)
    q = random_sphere_points(3000, seed=22)
    m = nat.Mesh(verts, tris, 4)
    cs = [m.assemble(dev(j)) for j in jets]
    out, _, _, jac = m.compose(cs, dev(q), want_jac=True)
    comp = OS.CompositeOracle(verts, tris, OG.ConeLocator(verts, tris), jets, tie_fix=True)
    X, J = OS.composite_jacobian(comp, q)
    J_gpu = host(jac)
    scale = np.abs(J).max(axis=(1, 2))[:, None, None]
    np.testing.assert_allclose(J_gpu / scale, J / scale, rtol=0, atol=1e-10)
    # tangent map: J q = 0 and X . J = 0
    assert np.abs(np.einsum("nij,nj->ni", J_gpu, q)).max() < 1e-12
    assert np.abs(np.einsum("ni,nij->nj", host(out), J_gpu)).max() < 1e-12
    # central differences along a tangent direction (away from edges)
    t = np.cross(q, [0.3, -0.5, 0.8])
    t /= np.linalg.norm(t, axis=1)[:, None]
    h = 1e-6
    qp = q + h * t
    qm = q - h * t
    qp /= np.linalg.norm(qp, axis=1)[:, None]
    qm /= np.linalg.norm(qm, axis=1)[:, None]
    fp, _, tap, _ = m.compose(cs, dev(qp), want_tri_all=True)
    fm, _, tam, _ = m.compose(cs, dev(qm), want_tri_all=True)
    same = (host(tap) == host(tam)).all(0)
    fd = (host(fp) - host(fm)) / (2 * h)
    an = np.einsum("nij,nj->ni", J_gpu, t)
    assert same.mean() > 0.9
    np.testing.assert_allclose(fd[same], an[same], rtol=0, atol=2e-6 * np.abs(an).max())


def test_edge_cases(nat):
    from cmm_gpu.meshgen import icosahedral_mesh
    verts, tris = icosahedral_mesh(2)
    m = nat.Mesh(verts, tris, 2)
    c = m.new_coeffs()
    empty = torch.empty((0, 3), dtype=torch.float64, device="cuda")
    out, tri, _, _ = m.compose([c], empty, want_tri=True)
    assert out.shape == (0, 3)
    q = dev(np.array([[np.nan, 0.0, 1.0], [0.0, 0.0, 1.0]]))
    tri, _ = m.locate(q)
    assert host(tri)[0] == -1
    assert m.status(clear=True) & nat.FLAG_NONFINITE
    assert m.status() == 0
    with pytest.raises(nat.CmmError) as e:
        m.compose([c] * 1025, dev(np.zeros((1, 3))))
    assert e.value.code == 1
    with pytest.raises(TypeError):
        m.locate(torch.zeros((3, 3)))
    # the poles and the 12 base vertices locate without a status flag
    q = dev(verts[[0, -1] + list(range(1, 11))])
    tri, bcc = m.locate(q)
    assert (host(tri) >= 0).all() and m.status() == 0


@pytest.mark.parametrize("level,n", [(2, 1000), (5, 70001), (6, 0)])
def test_ordered_compose_bitwise_equal(nat, level, n):
    """cmm_query_order gives a permutation grouped by coarse cell, and the
    composition processed in that order writes the same bits (points,
    triangles of every submap, Jacobians) as the caller-order composition."""
    from cmm_gpu.meshgen import icosahedral_mesh, random_sphere_points
    from cmm_gpu.workloads import submap_stack
    verts, tris = icosahedral_mesh(level)
    mesh = nat.Mesh(verts, tris, level)
    tan, s_pts = OG.stencil_points(verts)
    coeffs = [mesh.assemble(dev(j)) for j in submap_stack(s_pts, tan, 3, seed=5)]
    q = dev(random_sphere_points(n, seed=6)) if n else torch.empty((0, 3), dtype=torch.float64,
                                                                  device="cuda")
    perm = mesh.query_order(q)
    assert torch.equal(torch.sort(perm.long())[0], torch.arange(n, device="cuda"))
    a = mesh.compose(coeffs, q, want_tri=True, want_tri_all=True, want_jac=True)
    b = mesh.compose(coeffs, q, want_tri=True, want_tri_all=True, want_jac=True, perm=perm)
    for x, y in zip(a, b):
        assert torch.equal(x, y)
    if n and level >= 4:
        # neighbours in the order mostly share a level-4 cell (about 0.05
        # across), against a mean distance near 1.3 between random points
        pts = host(q)[host(perm)]
        step = np.linalg.norm(pts[1:] - pts[:-1], axis=1)
        assert np.median(step) < 0.1, np.median(step)
    assert mesh.status(clear=True) == 0


def test_full_size_composition_properties(nat):
    """The map-evaluation workload at full size (level 7, 8 submaps, 2^24
    queries, ids and Jacobians), through size-independent properties:
    images on the sphere; composing the stack in two launches (submaps 4-7,
    then 0-3) gives the same points to a few ulp (the second launch
    normalises its input point, which the single launch carries
    unnormalised through its deferred projection) and the chain-rule product
    of the two Jacobians (to 1e-10 relative: the tangent pushes run in
    float-float, ~2^-47 per operation, and each push cancels terms ~1/h =
    120 times larger than its result; measured 2.8e-11 over the 2^24
    queries); the ids of the first submap applied equal plain location; and
    a 4096-query sample matches the oracle (1e-12 points, 1e-10 relative
    Jacobians)."""
    from cmm_gpu.meshgen import icosahedral_mesh, random_sphere_points, stencil_frames
    from cmm_gpu.workloads import submap_stack
    verts, tris = icosahedral_mesh(7)
    tan, s_pts = stencil_frames(verts)
    jets = submap_stack(s_pts, tan, 8, seed=1)
    m = nat.Mesh(verts, tris, 7)
    cs = [m.assemble(dev(j)) for j in jets]
    q = dev(random_sphere_points(1 << 24, seed=3))
    X, tri, _, J = m.compose(cs, q, want_tri=True, want_jac=True)
    assert float((X.norm(dim=1) - 1).abs().max()) < 1e-15
    Y, _, _, JB = m.compose(cs[4:], q, want_jac=True)
    X2, _, _, JA = m.compose(cs[:4], Y, want_jac=True)
    assert float((X - X2).abs().max()) < 2e-15
    del X2, Y
    JJ = torch.bmm(JA, JB)
    del JA, JB
    rel = float(((JJ - J).abs().amax(dim=(1, 2)) / J.abs().amax(dim=(1, 2))).max())
    assert rel < 1e-10, rel
    del JJ
    t0, _ = m.locate(q)
    assert torch.equal(t0, tri)
    assert m.status() == 0
    # oracle on a sample
    idx = np.random.default_rng(0).choice(1 << 24, 4096, replace=False)
    qs = host(q[torch.from_numpy(idx).cuda()])
    comp = OS.CompositeOracle(verts, tris, OG.ConeLocator(verts, tris), jets, tie_fix=True)
    np.testing.assert_allclose(host(X)[idx], comp(qs), rtol=0, atol=1e-12)
    _, Jo = OS.composite_jacobian(comp, qs)
    Jg = host(J)[idx]
    scale = np.abs(Jo).max(axis=(1, 2))[:, None, None]
    np.testing.assert_allclose(Jg / scale, Jo / scale, rtol=0, atol=1e-10)
    # the same workload through map forms: ids equal, points within 1e-13
    fs = [m.assemble_forms(c) for c in cs]
    Xf, tf, _, Jf = m.compose(cs, q, want_tri=True, want_jac=True, forms=fs)
    assert torch.equal(tf, tri)
    assert float((Xf - X).abs().max()) < 1e-13
    assert float(((Jf - J).abs().amax(dim=(1, 2)) / J.abs().amax(dim=(1, 2))).max()) < 1e-10
    assert m.status() == 0


def test_ordered_compose_rejects_bad_permutation_entries(nat):
    """Entries outside [0, n) are skipped by the kernel's own bounds check and
    reported as CMM_FLAG_INDEX; every other query is composed as usual."""
    from cmm_gpu.meshgen import icosahedral_mesh, random_sphere_points
    from cmm_gpu.workloads import submap_stack
    verts, tris = icosahedral_mesh(3)
    mesh = nat.Mesh(verts, tris, 3)
    tan, s_pts = OG.stencil_points(verts)
    coeffs = [mesh.assemble(dev(j)) for j in submap_stack(s_pts, tan, 2, seed=5)]
    n = 1000
    q = dev(random_sphere_points(n, seed=8))
    perm = torch.arange(n, dtype=torch.int32, device="cuda")
    perm[3], perm[5] = n + 7, -2          # queries 3 and 5 are then never visited
    ref = mesh.compose(coeffs, q)[0]
    out = torch.full((n, 3), 7.0, dtype=torch.float64, device="cuda")
    mesh.compose(coeffs, q, out=out, perm=perm)
    assert mesh.status(clear=True) == nat.FLAG_INDEX
    keep = torch.ones(n, dtype=torch.bool, device="cuda")
    keep[[3, 5]] = False
    assert torch.equal(out[keep], ref[keep])
    assert bool((out[~keep] == 7.0).all())


def test_map_forms_match_coefficient_records(nat):
    """Composition through map-form records (cmm_assemble_forms /
    cmm_compose_forms: each Powell-Sabin patch as the quadratic form
    p^T Q p, FP32-filtered sub-triangle choice) against the same submaps'
    coefficient records and the oracle, level 5, 8 submaps, 2^16 queries:
    same triangle ids; points within 1e-13 of the records' and 1e-12 of the
    oracle's; Jacobians within 1e-11 (relative) of the records' and 1e-10
    of the oracle's; a stack mixing forms and records; the coarse-cell
    order bitwise equal to caller order."""
    from cmm_gpu.meshgen import icosahedral_mesh, random_sphere_points, stencil_frames
    from cmm_gpu.workloads import submap_stack
    verts, tris = icosahedral_mesh(5)
    tan, s_pts = stencil_frames(verts)
    jets = submap_stack(s_pts, tan, 8, seed=4)
    m = nat.Mesh(verts, tris, 5)
    cs = [m.assemble(dev(j)) for j in jets]
    fs = [m.assemble_forms(c) for c in cs]
    q = dev(random_sphere_points(1 << 16, seed=6))
    Xr, tr, tar, Jr = m.compose(cs, q, want_tri=True, want_tri_all=True, want_jac=True)
    Xf, tf, taf, Jf = m.compose(cs, q, want_tri=True, want_tri_all=True, want_jac=True, forms=fs)
    assert torch.equal(tr, tf) and torch.equal(tar, taf)
    assert float((Xf - Xr).abs().max()) < 1e-13
    scale = Jr.abs().amax(dim=(1, 2), keepdim=True)
    assert float(((Jf - Jr).abs() / scale).max()) < 1e-11
    Xm, _, _, Jm = m.compose(cs, q, want_jac=True, forms=[fs[0], None, fs[2], None, None, fs[5], fs[6], None])
    assert float((Xm - Xr).abs().max()) < 1e-13
    perm = m.query_order(q)
    Xo, to, _, Jo = m.compose(cs, q, want_tri=True, want_jac=True, forms=fs, perm=perm)
    assert torch.equal(Xo, Xf) and torch.equal(to, tf) and torch.equal(Jo, Jf)
    comp = OS.CompositeOracle(verts, tris, OG.ConeLocator(verts, tris), jets, tie_fix=True)
    qs = host(q)[:4096]
    np.testing.assert_allclose(host(Xf)[:4096], comp(qs), rtol=0, atol=1e-12)
    _, Jor = OS.composite_jacobian(comp, qs)
    sc = np.abs(Jor).max(axis=(1, 2))[:, None, None]
    np.testing.assert_allclose(host(Jf)[:4096] / sc, Jor / sc, rtol=0, atol=1e-10)
    # the low floats of the forms' float-float split (cmm_forms_ff): the
    # Jacobian pushes load the same floats they would extract, so every
    # output is bitwise the one without them, in both orders and in a
    # mixed stack
    gs = [m.forms_ff(f) for f in fs]
    assert gs[0].shape == (m.nt, nat.Mesh.FORM_FF_STRIDE) and gs[0].dtype == torch.float32
    assert bool((gs[0][:, 108:] == 0).all())
    Xg, tg, tag, Jg = m.compose(cs, q, want_tri=True, want_tri_all=True, want_jac=True, forms=fs, forms_ff=gs)
    assert torch.equal(Xg, Xf) and torch.equal(tg, tf) and torch.equal(tag, taf) and torch.equal(Jg, Jf)
    Xgo, _, _, Jgo = m.compose(cs, q, want_jac=True, forms=fs, forms_ff=gs, perm=perm)
    assert torch.equal(Xgo, Xf) and torch.equal(Jgo, Jf)
    mixed = [fs[0], None, fs[2], None, None, fs[5], fs[6], None]
    Xgm, _, _, Jgm = m.compose(cs, q, want_jac=True, forms=mixed,
                               forms_ff=[gs[0], None, gs[2], None, None, None, gs[6], None])
    assert torch.equal(Xgm, Xm) and torch.equal(Jgm, Jm)
    # non-finite queries through the forms path
    qn = q[:64].clone()
    qn[3, 1] = float("nan")
    Xn, tn, _, Jn = m.compose(cs, qn, want_tri=True, want_jac=True, forms=fs)
    assert torch.isnan(Xn[3]).all() and int(tn[3]) == -1 and torch.isfinite(Xn[4:]).all()
    assert m.status(clear=True) == nat.FLAG_NONFINITE
    assert m.status() == 0
