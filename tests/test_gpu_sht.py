"""GPU parity: MWSS transforms and the vorticity -> velocity-jet pipeline
against the oracle's restated transform and the reference's closed forms.

Tolerances: coefficients and samples within 1e-12 relative to their
largest magnitude; velocity jets within 1e-12 relative (values) and 1e-11
relative (gradients, which carry an extra factor ~L)."""
import os

import numpy as np
import pytest
import torch

from conftest import GOLDEN
from oracle import sht as S
from oracle import geometry as OG

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def nat():
    import __graft_entry__
    __graft_entry__.build()
    from cmm_gpu import native
    return native


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def mhalf(a_lm):
    """oracle (L,L) [l,m] -> device layout [m,l]."""
    return np.ascontiguousarray(a_lm.T)


@pytest.mark.parametrize("L", [8, 32, 128])
def test_forward_matches_oracle_on_generic_samples(nat, L):
    rng = np.random.default_rng(L)
    f = rng.standard_normal((L + 1, 2 * L))
    f[0] = f[0, 0]   # the poles are single points
    f[-1] = f[-1, 0]
    ref = S.MWSS(L).forward(f)
    got = nat.Sht(L).forward(dev(f)).cpu().numpy()
    scale = np.abs(ref).max()
    np.testing.assert_allclose(got / scale, mhalf(ref) / scale, rtol=0, atol=1e-12)


@pytest.mark.parametrize("L", [8, 64])
def test_inverse_matches_oracle(nat, L):
    rng = np.random.default_rng(L + 1)
    a = np.tril(rng.standard_normal((L, L)) + 1j * rng.standard_normal((L, L)))
    a[:, 0] = a[:, 0].real
    ref = S.MWSS(L).inverse(a)
    sht = nat.Sht(L)
    got = sht.inverse(dev(mhalf(a))).cpu().numpy()
    scale = np.abs(ref).max()
    np.testing.assert_allclose(got / scale, ref / scale, rtol=0, atol=1e-12)
    many = np.stack([mhalf(a * (k + 1)) for k in range(12)])
    got12 = sht.inverse(dev(many)).cpu().numpy()
    for k in range(12):
        np.testing.assert_allclose(got12[k] / scale, (k + 1) * ref / scale, rtol=0, atol=1e-12)


def grid(L):
    from cmm_gpu.meshgen import latlon_mesh_arrays
    theta, phi, g, verts = latlon_mesh_arrays(L)
    Phi, The = np.meshgrid(phi, theta)
    return theta, phi, g, verts, Phi, The


def test_velocity_jets_match_reference_fixture(nat):
    """The fixture's velocity levels came from the reference's project_stream
    (with the restated transform standing in for pyssht)."""
    d = np.load(os.path.join(GOLDEN, "velocity_L8.npz"))
    L = 8
    theta, phi, g, verts, Phi, The = grid(L)
    vm = nat.VelMesh(L, theta, phi, g, verts)
    sht = nat.Sht(L)
    for n, t in enumerate([0.0, 0.1, 0.2]):
        om = (30 * np.cos(The) * np.cos(4 * (Phi + 2 * 2 * np.pi * t / 30)) * np.sin(The) ** 4
              + 0.3 * np.sin(The) ** 2 * np.cos(2 * Phi + t))
        jets = sht.velocity(vm, dev(om)).cpu().numpy()
        ref = d["vals"][n]
        s = np.abs(ref).max(axis=(1, 2), keepdims=True)
        np.testing.assert_allclose(jets[:, :1] / s, ref[:, :1] / s, rtol=0, atol=1e-12)
        np.testing.assert_allclose(jets[:, 1:] / s, ref[:, 1:] / s, rtol=0, atol=1e-11)


@pytest.mark.parametrize("L", [64, 256, 1024])
def test_rossby_haurwitz_velocity_closed_form(nat, L):
    """cmm_s2/tests/test_spherical_harmonic_tools.py:48-61 closed forms."""
    theta, phi, g, verts, Phi, The = grid(L)
    vm = nat.VelMesh(L, theta, phi, g, verts)
    om = 30 * np.cos(The) * np.cos(4 * Phi) * np.sin(The) ** 4
    jets = nat.Sht(L).velocity(vm, dev(om)).cpu().numpy()
    x, y, z = [c.reshape(-1) for c in g]
    psi_x = -32 * z * x ** 3 + 16 * z * (1 - z ** 2) * x
    psi_z = -(1 - z ** 2) ** 2 + 4 * z ** 2 * (1 - z ** 2) + 8 * x ** 2 * (1 - 3 * z ** 2) - 8 * x ** 4
    vel = np.array([y * psi_z, z * psi_x - x * psi_z, -y * psi_x]).reshape(3, L + 1, 2 * L)
    ref = np.concatenate([vel[:, 0, :1], vel[:, 1:-1].reshape(3, -1), vel[:, -1, :1]], 1)
    assert np.abs(jets[:, 0] - ref).max() < 1e-12


def test_velocity_generic_against_oracle(nat):
    L = 48
    theta, phi, g, verts, Phi, The = grid(L)
    rng = np.random.default_rng(5)
    om = np.exp(-((np.cos(The) - 0.3) ** 2) / 0.05) * np.cos(3 * Phi) + 0.1 * rng.standard_normal(Phi.shape)
    om[0] = om[0, 0]
    om[-1] = om[-1, 0]
    vm = nat.VelMesh(L, theta, phi, g, verts)
    jets = nat.Sht(L).velocity(vm, dev(om)).cpu().numpy()
    sht = S.MWSS(L)
    lp, lm, lz = S.ladder_operators(L)
    psi = S.inv_laplacian(om, sht, S.inverse_laplacian_diag(L))
    ref = S.velocity_jets(psi, sht, g, lp, lm, lz)
    s = np.abs(ref).max(axis=(1, 2), keepdims=True)
    np.testing.assert_allclose(jets / s, ref / s, rtol=0, atol=1e-11)


def test_scalar_spline_route_matches_reference(nat):
    """cmm_sht_scalar_jets + cmm_assemble(ncomp=1) + the spline term of
    cmm_vorticity_eval against the reference's project_onto_S12 fixture."""
    from oracle import spline as OSP
    d = np.load(os.path.join(GOLDEN, "scalar_L8.npz"))
    L = 8
    theta, phi, g, verts, Phi, The = grid(L)
    vm = nat.VelMesh(L, theta, phi, g, verts)
    sht = nat.Sht(L)
    jets = sht.scalar_jets(vm, dev(mhalf(d["alm_half"]))).cpu().numpy()
    np.testing.assert_allclose(jets, d["vals"], rtol=0, atol=1e-12)
    co = vm.assemble(dev(jets))
    rec = co.cpu().numpy()[:, :19].T
    np.testing.assert_allclose(rec, d["coeffs"], rtol=0, atol=1e-12)
    rng = np.random.default_rng(3)
    X = rng.standard_normal(((L + 1) * 2 * L, 3))
    X /= np.linalg.norm(X, axis=1)[:, None]
    om = vm.vorticity(nat.VORT_NONE, [], dev(X), 0.0, spline=co).cpu().numpy().reshape(-1)
    mu = OG.LatLonMesh(L)
    bcc, tri, vs = mu.query(X)
    ref = OSP.eval_patch(d["coeffs"], tri, bcc, vs, X)
    np.testing.assert_allclose(om, ref, rtol=0, atol=1e-12)


@pytest.mark.parametrize("schedule", [0, 1])
@pytest.mark.parametrize("L", [32, 128, 256, 1024])
def test_split_bf16_synthesis_against_fp64(nat, L, schedule):
    """The 12-field synthesis on the tensor cores (three bf16 products,
    FP32 per 64-degree chunk, compensated FP32 across chunks) against the
    FP64 path, up to the band-limit of the large configuration.  Measured
    5.0e-6..5.8e-6 of max |fp64| per field; asserted below 2e-5 (each split
    factor carries ~2^-17 relative error).  Both synthesis schedules: per
    chunk drained into compensated sums by the same warps (0), and
    warp-specialised (1), where copy, MMA and drain warps run concurrently."""
    rng = np.random.default_rng(L)
    a = np.zeros((12, L, L), dtype=complex)
    for f in range(12):
        c = np.tril(rng.standard_normal((L, L)) + 1j * rng.standard_normal((L, L)))
        c[:, 0] = c[:, 0].real
        a[f] = mhalf(c / (1 + np.arange(L))[:, None])
    ref = nat.Sht(L).inverse(dev(a)).cpu().numpy()
    tc = nat.Sht(L).set_schedule(schedule).set_precision(nat.Sht.SPLIT_BF16)
    got = tc.inverse(dev(a)).cpu().numpy()
    assert tc.status() == 0
    err = np.abs(got - ref).max(axis=(1, 2)) / np.abs(ref).max(axis=(1, 2))
    print(f"L={L} schedule {schedule}: split-BF16 synthesis relative error per field max {err.max():.3e}")
    assert err.max() < 2e-5
    assert err.max() > 1e-9   # the tensor-core path really ran (not FP64)


@pytest.mark.parametrize("L", [128, 1024])
def test_split_bf16_synthesis_schedules_bitwise_equal(nat, L):
    """Both synthesis schedules issue the same products per 64-degree chunk
    and add the chunk partials into the same compensated FP32 sums in the
    same order: their spectra, and so the synthesised fields, are bitwise
    equal."""
    rng = np.random.default_rng(7 + L)
    a = np.zeros((12, L, L), dtype=complex)
    for f in range(12):
        c = np.tril(rng.standard_normal((L, L)) + 1j * rng.standard_normal((L, L)))
        c[:, 0] = c[:, 0].real
        a[f] = mhalf(c / (1 + np.arange(L))[:, None])
    outs = []
    for schedule in (0, 1):
        tc = nat.Sht(L).set_schedule(schedule).set_precision(nat.Sht.SPLIT_BF16)
        outs.append(tc.inverse(dev(a)))
        assert tc.status() == 0
    assert torch.equal(outs[0], outs[1])


@pytest.mark.parametrize("L,n", [(33, 3), (128, 8), (1024, 4)])
def test_batched_analysis_bitwise_equal(nat, L, n):
    """Up to 8 split-BF16 plans of one band-limit (sharing the owner's
    tables) whose analyses run as one tensor-core launch, member b in
    columns 2b, 2b+1 of the N = 16 data tiles (cmm_sht_batch_forward):
    each member's coefficients are bitwise its own plan's."""
    rng = np.random.default_rng(50 + L)
    owner = nat.Sht(L).set_precision(nat.Sht.SPLIT_BF16)
    plans = [owner] + [nat.Sht(L).share_tables(owner) for _ in range(n - 1)]
    fs = []
    for _ in range(n):
        f = rng.standard_normal((L + 1, 2 * L))
        f[0], f[-1] = f[0, 0], f[-1, 0]
        fs.append(dev(f))
    batch = nat.ShtBatch(plans)
    got = batch.forward(fs)
    for b in range(n):
        assert torch.equal(got[b], plans[b].forward(fs[b])), b
    assert all(p.status() == 0 for p in plans)
    # every member must be a distinct split-BF16 plan of the batch's
    # band-limit, in no other batch
    with pytest.raises(RuntimeError):
        nat.ShtBatch([owner])
    with pytest.raises(RuntimeError):
        nat.ShtBatch([nat.Sht(L).share_tables(owner), nat.Sht(L)])
    del batch
    other = nat.ShtBatch(plans[:2])   # free again once the batch is gone
    del other


@pytest.mark.parametrize("L", [33, 128, 256])
def test_split_bf16_analysis_against_fp64(nat, L):
    """The forward Legendre analysis on the tensor cores (M = 128 degrees,
    K = 64 fine ring pairs per chunk, weights folded into the data tiles)
    against the FP64 path on generic samples.  Measured 3.4e-6..3.8e-6 of
    max |fp64|; asserted below 1.5e-5."""
    rng = np.random.default_rng(1000 + L)
    f = rng.standard_normal((L + 1, 2 * L))
    f[0] = f[0, 0]
    f[-1] = f[-1, 0]
    ref = nat.Sht(L).forward(dev(f)).cpu().numpy()
    tc = nat.Sht(L).set_precision(nat.Sht.SPLIT_BF16)
    got = tc.forward(dev(f)).cpu().numpy()
    assert tc.status() == 0
    low = np.tril(np.ones((L, L), dtype=bool)).T   # [m, l] entries with l >= m
    err = np.abs(got - ref)[low].max() / np.abs(ref[low]).max()
    print(f"L={L}: split-BF16 analysis relative error {err:.3e}")
    assert err < 1.5e-5
    assert err > 1e-9


@pytest.mark.parametrize("L", [128, 1024])
def test_split_bf16_velocity_jets(nat, L):
    """The whole velocity pipeline (analysis, D^-1, ladders, 12-field
    synthesis, jets) in the split-BF16 form against the FP64 form, up to
    the band-limit of the large configuration.  Measured ~9e-6 of the
    largest jet value; asserted below 3e-5."""
    theta, phi, g, verts, Phi, The = grid(L)
    vm = nat.VelMesh(L, theta, phi, g, verts)
    om = 30 * np.cos(The) * np.cos(4 * Phi) * np.sin(The) ** 4 + np.exp(-((np.cos(The) - 0.5) / 0.1) ** 2)
    ref = nat.Sht(L).velocity(vm, dev(om)).cpu().numpy()
    tc = nat.Sht(L).set_precision(nat.Sht.SPLIT_BF16)
    got = tc.velocity(vm, dev(om)).cpu().numpy()
    err = np.abs(got - ref).max() / np.abs(ref).max()
    print(f"L={L}: split-BF16 velocity jets relative error {err:.3e}")
    assert 1e-9 < err < 3e-5
    assert tc.status() == 0


def test_power_matches_energy_spectrum(nat):
    """cmm_sht_power against the oracle's energy_spectrum
    (core/spherical_harmonic_tools.py:157-163) of the same coefficients:
    power[0] = spectrum[0], power[l] = l (l+1) spectrum[l]; 1e-13 relative."""
    L = 48
    rng = np.random.default_rng(9)
    a = np.tril(rng.standard_normal((L, L)) + 1j * rng.standard_normal((L, L)))
    a[:, 0] = a[:, 0].real
    spec = S.energy_spectrum(S.shifted_from_vec(S.full_from_half(a), L))
    ell = np.arange(L)
    ref = spec * np.where(ell > 0, ell * (ell + 1), 1)
    got = nat.Sht(L).power(dev(mhalf(a))).cpu().numpy()
    np.testing.assert_allclose(got, ref, rtol=1e-13, atol=0)


@pytest.mark.parametrize("L", [8, 64, 300, 600])
def test_fp64_table_and_recurrence_stages_agree(nat, L):
    """The FP64 Legendre stages from Pbar tables (cmm_sht_set_tables) and from
    the on-the-fly recurrence give the same analysis, 12-field synthesis and
    velocity jets to rounding (1e-13 of the largest value); L = 600 forces
    the tables above their default range, L = 8..300 the recurrence below."""
    rng = np.random.default_rng(L + 7)
    f = rng.standard_normal((L + 1, 2 * L))
    f[0], f[-1] = f[0, 0], f[-1, 0]
    a = np.tril(rng.standard_normal((L, L)) + 1j * rng.standard_normal((L, L)))
    a[:, 0] = a[:, 0].real
    many = dev(np.stack([mhalf(a * (k + 1)) for k in range(12)]))
    out = {}
    for mode in (nat.Sht.TABLES_NEVER, nat.Sht.TABLES_ALWAYS):
        sht = nat.Sht(L).set_tables(mode)
        out[mode] = (sht.forward(dev(f)).cpu().numpy(), sht.inverse(many).cpu().numpy())
        assert sht.status() == 0
    for x, y in zip(out[nat.Sht.TABLES_NEVER], out[nat.Sht.TABLES_ALWAYS]):
        scale = np.abs(x).max()
        np.testing.assert_allclose(y / scale, x / scale, rtol=0, atol=1e-13)
    if L == 64:
        theta, phi, g, verts, Phi, The = grid(L)
        vm = nat.VelMesh(L, theta, phi, g, verts)
        om = np.cos(The) ** 3 * np.sin(2 * Phi) + 0.05 * rng.standard_normal(Phi.shape)
        om[0], om[-1] = om[0, 0], om[-1, 0]
        j0 = nat.Sht(L).set_tables(nat.Sht.TABLES_NEVER).velocity(vm, dev(om)).cpu().numpy()
        j1 = nat.Sht(L).velocity(vm, dev(om)).cpu().numpy()
        s = np.abs(j0).max()
        np.testing.assert_allclose(j1 / s, j0 / s, rtol=0, atol=1e-13)


def test_shared_fp64_tables_give_the_owners_bits(nat):
    """A plan on another plan's FP64 Pbar tables (cmm_sht_share_tables with
    an FP64 source) gives the bits of a plan with its own tables, also after
    the owner is trimmed (the tables live while a holder does); sharing from
    a plan that runs without tables, or from itself, is an argument error."""
    L = 48
    rng = np.random.default_rng(3)
    f = rng.standard_normal((L + 1, 2 * L))
    f[0], f[-1] = f[0, 0], f[-1, 0]
    a = np.tril(rng.standard_normal((L, L)) + 1j * rng.standard_normal((L, L)))
    a[:, 0] = a[:, 0].real
    many = dev(np.stack([mhalf(a * (k + 1)) for k in range(12)]))
    own = nat.Sht(L)
    ref = (own.forward(dev(f)), own.inverse(many))
    src = nat.Sht(L)
    user = nat.Sht(L).share_tables(src)
    src.trim()
    got = (user.forward(dev(f)), user.inverse(many))
    for x, y in zip(ref, got):
        assert torch.equal(x, y)
    assert user.status() == 0
    with pytest.raises(RuntimeError):
        nat.Sht(L).share_tables(nat.Sht(L).set_tables(nat.Sht.TABLES_NEVER))
    with pytest.raises(RuntimeError):
        user.share_tables(user)


def test_bounded_wait_timeout_sets_status_and_context_survives(nat):
    """The tensor-core kernels' bounded mbarrier wait, run on a barrier that
    nothing completes (cmm_sht_timeout_selftest, 1000 polls), runs out, sets
    CMM_FLAG_TIMEOUT in the plan's status word and returns; the context
    stays usable (a split-BF16 transform afterwards is still correct)."""
    L = 32
    tc = nat.Sht(L).set_precision(nat.Sht.SPLIT_BF16)
    assert tc.status() == 0
    tc.timeout_selftest(1000)
    assert tc.status(clear=True) == nat.FLAG_TIMEOUT
    assert tc.status() == 0
    f = np.random.default_rng(3).standard_normal((L + 1, 2 * L))
    f[0], f[-1] = f[0, 0], f[-1, 0]
    a64 = nat.Sht(L).forward(dev(f))
    a16 = tc.forward(dev(f))
    rel = float((a16 - a64).abs().max() / a64.abs().max())
    assert 1e-9 < rel < 1e-4 and tc.status() == 0


def test_full_size_round_trip_and_split_error(nat):
    """At the band-limit of the large configuration (L = 1024): a random
    band-limited field synthesised and analysed again comes back to 1e-12 of
    its largest coefficient in FP64 (the MWSS transform is exact for
    band-limited samples); the split-BF16 analysis of the same samples stays
    within 2e-5 (measured ~5e-6) and above 1e-9 (the tensor-core path
    ran)."""
    L = 1024
    rng = np.random.default_rng(11)
    a = np.tril(rng.standard_normal((L, L)) + 1j * rng.standard_normal((L, L)))
    a[:, 0] = a[:, 0].real
    ell = np.arange(L)[:, None] + 1.0
    a = a * ell ** -1.0                      # a decaying spectrum over all degrees
    sht = nat.Sht(L)
    f = sht.inverse(dev(mhalf(a)))
    back = sht.forward(f).cpu().numpy()
    scale = np.abs(a).max()
    np.testing.assert_allclose(back / scale, mhalf(a) / scale, rtol=0, atol=1e-12)
    tc = nat.Sht(L).set_precision(nat.Sht.SPLIT_BF16)
    b16 = tc.forward(f).cpu().numpy()
    err = np.abs(b16 - mhalf(a)).max() / scale
    assert 1e-9 < err < 2e-5, err
    assert tc.status() == 0 and sht.status() == 0


ORDERS_1024 = [0, 1, 2, 17, 255, 511, 512, 777, 1000, 1022, 1023]


def test_fp64_forward_matches_oracle_at_full_bandlimit(nat):
    """FP64 analysis at L = 1024 of generic (not band-limited) samples
    against the oracle's single-order restatement on a spread of orders m
    (the full oracle table would hold 17 GB): 1e-12 of the largest
    coefficient."""
    L = 1024
    rng = np.random.default_rng(1024)
    f = rng.standard_normal((L + 1, 2 * L))
    f[0], f[-1] = f[0, 0], f[-1, 0]
    got = nat.Sht(L).forward(dev(f)).cpu().numpy()           # [m, l]
    ref = S.forward_orders(f, L, ORDERS_1024)                # [k, l]
    scale = np.abs(ref).max()
    for k, m in enumerate(ORDERS_1024):
        np.testing.assert_allclose(got[m, m:] / scale, ref[k, m:] / scale, rtol=0, atol=1e-12)


def test_fp64_inverse_matches_oracle_at_full_bandlimit(nat):
    """FP64 synthesis at L = 1024 of coefficients on a spread of orders
    against the oracle's single-order restatement, every sample of the
    (1025, 2048) grid: 1e-12 of the largest sample."""
    L = 1024
    rng = np.random.default_rng(1025)
    cols = np.zeros((len(ORDERS_1024), L), dtype=complex)
    a = np.zeros((L, L), dtype=complex)                      # [m, l]
    for k, m in enumerate(ORDERS_1024):
        c = (rng.standard_normal(L - m) + 1j * rng.standard_normal(L - m)) / np.sqrt(1.0 + np.arange(m, L))
        if m == 0:
            c = c.real
        cols[k, m:] = c
        a[m, m:] = c
    ref = S.inverse_orders(L, cols, ORDERS_1024)
    got = nat.Sht(L).inverse(dev(a)).cpu().numpy()
    scale = np.abs(ref).max()
    np.testing.assert_allclose(got / scale, ref / scale, rtol=0, atol=1e-12)
