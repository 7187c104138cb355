"""The restated MWSS transform on the reference's closed-form test pairs
(cmm_s2/tests/test_spherical_harmonic_tools.py:17-61,
cmm_s2/tests/sht_speed_tests.py:19-26)."""
import numpy as np
import pytest

from oracle import sht as S
from oracle.geometry import sphere2cart, LatLonMesh


def grid(L):
    m = LatLonMesh(L)
    return np.meshgrid(m.phi, m.theta), m


@pytest.mark.parametrize("L,l", [(32, 8), (64, 30)])
def test_poisson_pair(L, l):
    (Ph, Th), _ = grid(L)
    src = (l * (l + 1) + (l + 1) * (l + 2) * np.cos(Th)) * np.cos(l * Ph) * np.sin(Th) ** l
    sol = -(np.sin(Th) ** l) * np.cos(l * Ph) - np.cos(Th) * (np.sin(Th) ** l) * np.cos(l * Ph)
    sht = S.MWSS(L)
    rec = sht.inverse(sht.forward(src) * S.inverse_laplacian_diag(L)[:, None])
    assert np.abs(rec - sol).max() < 1e-12


@pytest.mark.parametrize("L", [16, 48])
def test_rossby_haurwitz_velocity(L):
    (Ph, Th), mesh = grid(L)
    omega = 30 * np.cos(Th) * np.cos(4 * Ph) * np.sin(Th) ** 4
    sht = S.MWSS(L)
    lp, lm, lz = S.ladder_operators(L)
    psi = S.inv_laplacian(omega, sht, S.inverse_laplacian_diag(L))
    vals = S.velocity_jets(psi, sht, mesh.grid_points, lp, lm, lz)
    x, y, z = [c.reshape(-1) for c in sphere2cart(Ph, Th)]
    psi_x = -32 * z * x ** 3 + 16 * z * (1 - z ** 2) * x
    psi_z = -(1 - z ** 2) ** 2 + 4 * z ** 2 * (1 - z ** 2) + 8 * x ** 2 * (1 - 3 * z ** 2) - 8 * x ** 4
    vel = np.array([y * psi_z, z * psi_x - x * psi_z, -y * psi_x]).reshape(3, L + 1, 2 * L)
    ref = np.concatenate([vel[:, 0, :1], vel[:, 1:-1].reshape(3, -1), vel[:, -1, :1]], 1)
    assert np.abs(vals[:, 0] - ref).max() < 1e-13


def test_bandlimited_round_trip():
    L = 40
    rng = np.random.default_rng(1)
    a = np.tril(rng.standard_normal((L, L)) + 1j * rng.standard_normal((L, L)))
    a[:, 0] = a[:, 0].real
    sht = S.MWSS(L)
    assert np.abs(sht.forward(sht.inverse(a)) - a).max() < 1e-13


def test_layout_round_trips():
    L = 9
    rng = np.random.default_rng(2)
    a = np.tril(rng.standard_normal((L, L)) + 1j * rng.standard_normal((L, L)))
    a[:, 0] = a[:, 0].real
    v = S.full_from_half(a)
    np.testing.assert_array_equal(S.half_from_full(v, L), a)
    np.testing.assert_array_equal(S.vec_from_shifted(S.shifted_from_vec(v, L), L), v)


def test_single_order_transforms_match_full_tables():
    """The per-order forms used at L = 1024 (where the full Legendre table
    would hold 17 GB) against the full-table transforms at L = 64."""
    L = 64
    ms = [0, 1, 5, 31, 63]
    rng = np.random.default_rng(8)
    f = rng.standard_normal((L + 1, 2 * L))
    f[0], f[-1] = f[0, 0], f[-1, 0]
    sht = S.MWSS(L)
    full = sht.forward(f)
    part = S.forward_orders(f, L, ms)
    for k, m in enumerate(ms):
        np.testing.assert_allclose(part[k], full[:, m], rtol=0, atol=1e-14 * np.abs(full).max())
    a = np.zeros((L, L), dtype=complex)
    cols = np.zeros((len(ms), L), dtype=complex)
    for k, m in enumerate(ms):
        cols[k, m:] = rng.standard_normal(L - m) + 1j * rng.standard_normal(L - m)
        if m == 0:
            cols[k] = cols[k].real
        a[:, m] = cols[k]
    ref = sht.inverse(a)
    np.testing.assert_allclose(S.inverse_orders(L, cols, ms), ref, rtol=0, atol=1e-13 * np.abs(ref).max())
