"""MWSS spherical-harmonic transforms and coefficient-space operators
(oracle).

The reference calls ``pyssht.forward/inverse(..., Method="MWSS",
Reality=True)`` (cmm_s2/core/spherical_harmonic_tools.py:16, 84, 91).  That
third-party package (ssht C library with the ducc0 backend; the reference
pins no version) is absent, so the transforms are restated here from the
published MW symmetric sampling theorem (McEwen & Wiaux 2011, IEEE TSP 59;
symmetric variant in Ocampo, Price & McEwen 2016):

* samples on MWSS rings theta_t = pi t / L (t = 0..L, both poles) and
  phi_p = 2 pi p / (2L);
* orthonormal Y_lm = Pbar_lm(theta) e^{i m phi} with the Condon-Shortley
  phase (the convention the reference's Rossby-Haurwitz closed forms
  require);
* inverse: evaluate the sum on the rings, then an inverse FFT in phi;
* forward: FFT in phi; extend each Fourier column to the theta-torus with
  F_m(2 pi - theta) = (-1)^m F_m(theta); take the trigonometric interpolant
  of the 2L torus samples (Nyquist term split evenly between +-L); integrate
  it exactly against Pbar_lm(theta) sin(theta) over [0, pi].  The exact
  integral is evaluated by resampling the interpolant on 2L+1 equispaced
  rings and applying Clenshaw-Curtis weights in x = cos(theta) (exact for
  the degree <= 2L-1 products).  For band-limited samples this equals every
  exact MWSS forward transform; for other inputs it is the MW construction
  (interpolate on the torus, integrate exactly) with the Nyquist convention
  stated above, so parity with pyssht on non-band-limited data is unpinned.

Coefficient layouts follow the reference: ``lm_vec`` index l*l + l + m
(pyssht.elm2ind) and the (L, 2L+1) "shifted" array with column m + l
(coeff_array / lm_array, cmm_s2/core/spherical_harmonic_tools.py:30-47).
"""
import numpy as np


def legendre_table(L, theta):
    """Pbar_lm(theta) for 0 <= m <= l < L: array (L, L, len(theta)) [l, m, j].

    Standard three-term recurrence in l from the sectoral start
    Pbar_mm = (-1)^m sqrt((2m+1)/(4 pi) prod_{k<=m} (2k-1)/(2k)) sin^m."""
    theta = np.asarray(theta, dtype=np.float64)
    x, s = np.cos(theta), np.sin(theta)
    P = np.zeros((L, L, len(theta)))
    pmm = np.full(len(theta), np.sqrt(1 / (4 * np.pi)))
    for m in range(L):
        if m > 0:
            pmm = -pmm * np.sqrt((2 * m + 1) / (2 * m)) * s
        P[m, m] = pmm
        if m + 1 < L:
            P[m + 1, m] = np.sqrt(2 * m + 3) * x * pmm
        for l in range(m + 2, L):
            a = np.sqrt((4 * l * l - 1) / (l * l - m * m))
            b = np.sqrt(((l - 1) ** 2 - m * m) / (4 * (l - 1) ** 2 - 1))
            P[l, m] = a * (x * P[l - 1, m] - b * P[l - 2, m])
    return P


def clenshaw_curtis(M):
    """Weights for int_{-1}^{1} g(x) dx at x_j = cos(pi j / M), j = 0..M (M even)."""
    j = np.arange(M + 1)
    w = np.ones(M + 1)
    for k in range(1, M // 2 + 1):
        b = 1.0 if k == M // 2 else 2.0
        w -= b / (4 * k * k - 1) * np.cos(2 * np.pi * j * k / M)
    c = np.full(M + 1, 2.0)
    c[0] = c[-1] = 1.0
    return c / M * w


class MWSS:
    """Real MWSS transforms at band-limit L (coefficients for m >= 0 only,
    array (L, L) indexed [l, m], zero for m > l)."""

    def __init__(self, L):
        self.L = L
        self.theta = np.pi * np.arange(L + 1) / L
        self.theta_fine = np.pi * np.arange(2 * L + 1) / (2 * L)
        self.P = legendre_table(L, self.theta)
        self.Pf = legendre_table(L, self.theta_fine)
        self.w = clenshaw_curtis(2 * L)

    def inverse(self, alm):
        """(L,L) complex [l,m>=0] -> real samples (L+1, 2L)."""
        L = self.L
        F = np.einsum("lm,lmt->tm", alm, self.P)            # (L+1, L)
        c = np.zeros((L + 1, L + 1), dtype=complex)
        c[:, :L] = F
        return np.fft.irfft(c, n=2 * L, axis=1) * (2 * L)

    def forward(self, f):
        """real samples (L+1, 2L) -> (L,L) complex [l, m>=0]."""
        L = self.L
        Fm = np.fft.rfft(f, axis=1)[:, :L] * (np.pi / L)   # int f e^{-im phi} dphi
        sign = (-1.0) ** np.arange(L)
        G = np.empty((2 * L, L), dtype=complex)
        G[:L + 1] = Fm
        G[L + 1:] = sign * Fm[L - 1:0:-1]
        Gh = np.fft.fft(G, axis=0) / (2 * L)
        H = np.zeros((4 * L, L), dtype=complex)
        H[:L] = Gh[:L]
        H[3 * L + 1:] = Gh[L + 1:]
        H[L] = Gh[L] / 2
        H[3 * L] = Gh[L] / 2
        fine = np.fft.ifft(H, axis=0)[:2 * L + 1] * (4 * L)  # interpolant on 2L+1 rings
        return np.einsum("jm,lmj,j->lm", fine, self.Pf, self.w)


# --------------------------------------------- single orders at large L
def legendre_m(L, m, theta):
    """Pbar_lm(theta) of one order m for m <= l < L: array (L, len(theta)),
    rows l < m zero; the recurrence of legendre_table for that column only
    (legendre_table(L) itself holds L^2 len(theta) values: 17 GB at L =
    1024)."""
    theta = np.asarray(theta, dtype=np.float64)
    x, s = np.cos(theta), np.sin(theta)
    P = np.zeros((L, len(theta)))
    pmm = np.full(len(theta), np.sqrt(1 / (4 * np.pi)))
    for k in range(1, m + 1):
        pmm = -pmm * np.sqrt((2 * k + 1) / (2 * k)) * s
    P[m] = pmm
    if m + 1 < L:
        P[m + 1] = np.sqrt(2 * m + 3) * x * pmm
    for l in range(m + 2, L):
        a = np.sqrt((4 * l * l - 1) / (l * l - m * m))
        b = np.sqrt(((l - 1) ** 2 - m * m) / (4 * (l - 1) ** 2 - 1))
        P[l] = a * (x * P[l - 1] - b * P[l - 2])
    return P


def inverse_orders(L, cols, ms):
    """MWSS.inverse of coefficients that are zero outside the orders ms:
    cols (len(ms), L) complex [k, l] holds a_{l, ms[k]}; real samples
    (L+1, 2L)."""
    theta = np.pi * np.arange(L + 1) / L
    c = np.zeros((L + 1, L + 1), dtype=complex)
    for k, m in enumerate(ms):
        c[:, m] = cols[k] @ legendre_m(L, m, theta)
    return np.fft.irfft(c, n=2 * L, axis=1) * (2 * L)


def forward_orders(f, L, ms):
    """MWSS.forward of the real samples f (L+1, 2L), the columns m in ms
    only: (len(ms), L) complex [k, l] = a_{l, ms[k]}."""
    ms = list(ms)
    Fm = np.fft.rfft(f, axis=1)[:, ms] * (np.pi / L)
    sign = (-1.0) ** np.asarray(ms)
    G = np.empty((2 * L, len(ms)), dtype=complex)
    G[:L + 1] = Fm
    G[L + 1:] = sign * Fm[L - 1:0:-1]
    Gh = np.fft.fft(G, axis=0) / (2 * L)
    H = np.zeros((4 * L, len(ms)), dtype=complex)
    H[:L] = Gh[:L]
    H[3 * L + 1:] = Gh[L + 1:]
    H[L] = Gh[L] / 2
    H[3 * L] = Gh[L] / 2
    fine = np.fft.ifft(H, axis=0)[:2 * L + 1] * (4 * L)
    w = clenshaw_curtis(2 * L)
    theta_fine = np.pi * np.arange(2 * L + 1) / (2 * L)
    return np.stack([legendre_m(L, m, theta_fine) @ (fine[:, k] * w) for k, m in enumerate(ms)])


# ------------------------------------------------------ coefficient layouts
def full_from_half(alm):
    """(L,L) m>=0 -> pyssht 1-D vector (L*L,) using a_{l,-m} = (-1)^m conj(a_lm)."""
    L = alm.shape[0]
    out = np.zeros(L * L, dtype=complex)
    for l in range(L):
        for m in range(-l, l + 1):
            out[l * l + l + m] = alm[l, m] if m >= 0 else (-1) ** m * np.conj(alm[l, -m])
    return out


def half_from_full(flm, L):
    out = np.zeros((L, L), dtype=complex)
    for l in range(L):
        out[l, :l + 1] = flm[l * l + l: l * l + 2 * l + 1]
    return out


def shifted_from_vec(flm, L):
    """coeff_array (cmm_s2/core/spherical_harmonic_tools.py:30-42)."""
    out = np.zeros((L, 2 * L + 1), dtype=complex)
    for l in range(L):
        out[l, :2 * l + 1] = flm[l * l: l * l + 2 * l + 1]
    return out


def vec_from_shifted(c, L):
    """lm_array (cmm_s2/core/spherical_harmonic_tools.py:44-47)."""
    return np.concatenate([c[l, :2 * l + 1] for l in range(L)])


def ladder_operators(L):
    """L_plus, L_minus, L_z in the shifted layout
    (cmm_s2/core/spherical_simulations.py:201-205)."""
    l = np.arange(L)[:, None].astype(np.float64)
    m = np.arange(2 * L + 1)[None, :] - l
    with np.errstate(invalid="ignore"):
        lp = np.sqrt(l * (l + 1) - m * (m - 1))
        lm = np.sqrt(l * (l + 1) - m * (m + 1))
    lp[np.isnan(lp)] = 0.0
    lm[np.isnan(lm)] = 0.0
    return lp, lm, np.broadcast_to(m, (L, 2 * L + 1)).copy()


def inverse_laplacian_diag(L):
    """D_inv (cmm_s2/core/spherical_simulations.py:195-198)."""
    els = np.arange(L)
    els[0] = 1
    d = -1 / (els * (els + 1))
    d[0] = 0.0
    return d


def angular_momentum(alms, lp, lm, lz):
    """i(L_x, L_y, L_z) on the shifted layout
    (cmm_s2/core/spherical_harmonic_tools.py:49-62)."""
    t = np.zeros_like(alms)
    t[:, 1:] = alms[:, :-1]
    up = lp * t
    t = np.zeros_like(alms)
    t[:, :-1] = alms[:, 1:]
    dn = lm * t
    ox = (up + dn) / 2
    oy = 1j * (dn - up) / 2
    return [1j * ox, 1j * oy, 1j * (lz * alms)]


def velocity_jets(psi_shifted, sht, grid_points, lp, lm, lz):
    """project_stream's spatial part (cmm_s2/core/spherical_harmonic_tools.py:78-101):
    velocity jets (3,4,Nv_u) on the lat-lon mesh vertices from the stream
    function in the shifted layout."""
    L = sht.L
    nv = 2 + (L - 1) * 2 * L
    vals = np.zeros((3, 4, nv))
    X = grid_points
    u = angular_momentum(psi_shifted, lp, lm, lz)

    def synth(c):
        return sht.inverse(half_from_full(vec_from_shifted(c, L), L))

    def put(dst, field):
        dst[1:-1] = field[1:-1].reshape((L - 1) * 2 * L)
        dst[-1] = field[-1, 0]
        dst[0] = field[0, 0]

    for i in range(3):
        put(vals[i, 0], synth(u[i]))
        g = angular_momentum(u[i], lp, lm, lz)
        G = [synth(gk) for gk in g]
        cr = [G[1] * X[2] - G[2] * X[1], G[2] * X[0] - G[0] * X[2], G[0] * X[1] - G[1] * X[0]]
        sc = (cr[0] * X[0] + cr[1] * X[1] + cr[2] * X[2]) / np.sqrt(X[0] ** 2 + X[1] ** 2 + X[2] ** 2)
        tp = [cr[k] - sc * X[k] for k in range(3)]
        for c in range(3):
            put(vals[c, 1 + i], tp[c])
    return vals


def scalar_jets(alm_half, sht, grid_points, lp, lm, lz):
    """project_onto_S12 (cmm_s2/core/spherical_harmonic_tools.py:108-142):
    jets (4,Nv_u) of the field with coefficients alm_half (L,L) [l,m>=0]:
    value from the inverse transform, gradient from the angular-momentum
    operators, g x X tangent-projected, poles from sample 0."""
    L = sht.L
    nv = 2 + (L - 1) * 2 * L
    vals = np.zeros((4, nv))
    X = grid_points
    c = shifted_from_vec(full_from_half(alm_half), L)

    def synth(ci):
        return sht.inverse(half_from_full(vec_from_shifted(ci, L), L))

    def put(dst, field):
        dst[1:-1] = field[1:-1].reshape((L - 1) * 2 * L)
        dst[-1] = field[-1, 0]
        dst[0] = field[0, 0]

    G = [synth(gk) for gk in angular_momentum(c, lp, lm, lz)]
    cr = [G[1] * X[2] - G[2] * X[1], G[2] * X[0] - G[0] * X[2], G[0] * X[1] - G[1] * X[0]]
    sc = (cr[0] * X[0] + cr[1] * X[1] + cr[2] * X[2]) / np.sqrt(X[0] ** 2 + X[1] ** 2 + X[2] ** 2)
    for k in range(3):
        put(vals[1 + k], cr[k] - sc * X[k])
    put(vals[0], synth(c))
    return vals


def inv_laplacian(samples, sht, dinv):
    """inv_Laplacian (cmm_s2/core/spherical_harmonic_tools.py:14-19): shifted layout."""
    L = sht.L
    return shifted_from_vec(full_from_half(sht.forward(samples)), L) * dinv[:, None]


def energy_spectrum(alms_shifted):
    """energy_spectrum (cmm_s2/core/spherical_harmonic_tools.py:157-163)."""
    L = alms_shifted.shape[0]
    p = np.real(np.sum(alms_shifted * np.conj(alms_shifted), axis=1))
    out = p.copy()
    out[1:] = p[1:] / (np.arange(1, L) * np.arange(2, L + 1))
    return out
