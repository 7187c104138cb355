"""Host-side pieces of the adjoint (no GPU): the angular-momentum series
behind the vorticity gradient.  The tangent gradient of a real SH series
f at a unit point x must equal -x cross (iL f)(x); checked against centred
differences of a numpy evaluation of the series."""
import numpy as np


def sh_eval(a, x):
    """Real orthonormal series (column l+m; m>0 sqrt2 cos, m<0 sqrt2 sin) at unit points x (n,3)."""
    lmax = a.shape[0] - 1
    z = x[:, 2]
    s = np.sqrt(np.maximum(0.0, 1 - z * z))
    phi = np.arctan2(x[:, 1], x[:, 0])
    out = np.zeros(len(x))
    pmm = np.full(len(x), np.sqrt(1 / (4 * np.pi)))
    for m in range(lmax + 1):
        if m > 0:
            pmm = -pmm * np.sqrt((2 * m + 1) / (2 * m)) * s
        p1, p = np.zeros_like(z), pmm.copy()
        for l in range(m, lmax + 1):
            if l == m + 1:
                p1, p = p, np.sqrt(2 * m + 3.0) * z * pmm
            elif l > m + 1:
                aa = np.sqrt((4.0 * l * l - 1) / (l * l - m * m))
                bb = np.sqrt(((l - 1.0) ** 2 - m * m) / (4.0 * (l - 1) ** 2 - 1))
                p1, p = p, aa * (z * p - bb * p1)
            if m == 0:
                out += a[l, l] * p
            else:
                out += np.sqrt(2) * p * (a[l, l + m] * np.cos(m * phi) + a[l, l - m] * np.sin(m * phi))
    return out


def test_il_series_gives_the_tangent_gradient():
    import sys, os
    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "..", "cmm-s2_gb300"))
    from cmm_gpu.adjoint import il_series, real_to_complex, complex_to_real
    rng = np.random.default_rng(3)
    lmax = 7
    a = np.zeros((lmax + 1, 2 * lmax + 1))
    for l in range(lmax + 1):
        a[l, :2 * l + 1] = rng.standard_normal(2 * l + 1)
    np.testing.assert_allclose(complex_to_real(real_to_complex(a)), a, atol=1e-15)
    x = rng.standard_normal((200, 3))
    x /= np.linalg.norm(x, axis=1)[:, None]
    d = il_series(a)
    Lv = np.stack([sh_eval(d[k], x) for k in range(3)], 1)
    grad = -np.cross(x, Lv)
    h = 1e-6
    fd = np.zeros_like(x)
    for k in range(3):
        e = np.zeros(3)
        e[k] = 1
        xp = x + h * e
        xm = x - h * e
        fd[:, k] = (sh_eval(a, xp / np.linalg.norm(xp, axis=1)[:, None]) -
                    sh_eval(a, xm / np.linalg.norm(xm, axis=1)[:, None])) / (2 * h)
    fd -= (fd * x).sum(1)[:, None] * x   # tangent part
    assert np.abs(grad - fd).max() < 1e-7 * np.abs(fd).max()
