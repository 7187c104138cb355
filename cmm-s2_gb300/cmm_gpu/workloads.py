"""Seeded synthetic workloads (host side, numpy).

The reference benchmarks nothing itself; the workloads here follow the
configurations its users run: random-rotation submap stacks for the map
composition microbenchmark, random spherical-harmonic initial vorticity for
the barotropic runs.  Everything is deterministic in the seed.
"""
import numpy as np


def random_rotation(rng):
    q = rng.standard_normal(4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def smooth_map(R, amp, rng):
    """x -> normalise(R x + amp * P_T(h(x))) with a low-degree harmonic
    field h and P_T the tangent projection at R x."""
    k = rng.standard_normal((3, 3))
    ph = rng.uniform(0, 2 * np.pi, 3)

    def f(x):  # x (N,3)
        y = x @ R.T
        h = np.stack([np.sin(x @ k[i] + ph[i]) for i in range(3)], 1)
        h -= np.einsum("ni,ni->n", h, y)[:, None] * y
        z = y + amp * h
        return z / np.linalg.norm(z, axis=1)[:, None]
    return f


def jets_from_stencil_images(img, tan, eps=1e-5):
    """Jets (3,4,Nv) from the images of the 4 stencil points, the way the
    CMM builds them (cmm_s2/core/evolution_functions.py:90-113):
    value = normalised stencil mean, gradient = centred differences in the
    vertex tangent frame.  img (3,4,Nv), tan (2,Nv,3)."""
    nv = img.shape[2]
    jets = np.empty((3, 4, nv))
    m = (img[:, 0] + img[:, 1] + img[:, 2] + img[:, 3]) / 4
    n = np.sqrt(m[0] ** 2 + m[1] ** 2 + m[2] ** 2)
    jets[:, 0] = m / n
    d1 = (img[:, 1] - img[:, 0] + img[:, 3] - img[:, 2]) / (4 * eps)
    d2 = (img[:, 2] - img[:, 0] + img[:, 3] - img[:, 1]) / (4 * eps)
    for k in range(3):
        jets[:, 1 + k] = (d1[k][:, None] * tan[0] + d2[k][:, None] * tan[1]).T
    return jets


def submap_stack(s_pts, tan, n_submaps, seed, amp=1e-2):
    """Jets (S,3,4,Nv) of S submaps R_s x + amp * harmonic perturbation."""
    rng = np.random.default_rng(seed)
    out = []
    pts = np.transpose(s_pts, (1, 2, 0)).reshape(-1, 3)        # (4*Nv, 3)
    for _ in range(n_submaps):
        f = smooth_map(random_rotation(rng), amp, rng)
        img = f(pts).reshape(4, -1, 3).transpose(2, 0, 1)     # (3,4,Nv)
        out.append(jets_from_stencil_images(img, tan))
    return np.stack(out)


def real_to_complex_sh(a, L):
    """Real orthonormal coefficients a (lmax+1, 2lmax+1) (column l+m; m>0 ->
    sqrt2 Pbar cos(m phi), m<0 -> sqrt2 Pbar sin(|m| phi)) -> complex
    coefficients of the transforms, m-major half layout (L, L) [m, l]:
    c_l0 = a_l0, c_lm = (a_{l,m} - i a_{l,-m}) / sqrt2."""
    lmax = a.shape[0] - 1
    out = np.zeros((L, L), dtype=np.complex128)
    for l in range(min(lmax + 1, L)):
        out[0, l] = a[l, l]
        for m in range(1, l + 1):
            out[m, l] = (a[l, l + m] - 1j * a[l, l - m]) / np.sqrt(2)
    return out


def spectral_perturbation(lmax, seed, slope=-2.0, rms=None):
    """Real SH coefficients a_lm ~ N(0,1) l^slope for 1 <= l <= lmax
    (slope -2 gives an energy spectrum sum_m a_lm^2 ~ l^-3), scaled to the
    given root-mean-square over the sphere when rms is set."""
    rng = np.random.default_rng(seed)
    a = np.zeros((lmax + 1, 2 * lmax + 1))
    for l in range(1, lmax + 1):
        a[l, :2 * l + 1] = rng.standard_normal(2 * l + 1) * float(l) ** slope
    if rms is not None:
        a *= rms / np.sqrt(np.sum(a ** 2) / (4 * np.pi))
    return a


def random_sh_vorticity(L_max, seed, slope=-1.5):
    """omega0(phi, theta) = sum_{l=1..L_max} sum_m a_lm Y^real_lm, a_lm ~ N(0,1) l^slope.

    Real orthonormal harmonics built from the same Pbar_lm as the transforms;
    returns (callable, coefficient array (L_max+1, 2*L_max+1))."""
    rng = np.random.default_rng(seed)
    a = np.zeros((L_max + 1, 2 * L_max + 1))
    for l in range(1, L_max + 1):
        a[l, :2 * l + 1] = rng.standard_normal(2 * l + 1) * float(l) ** slope

    def omega(phi, theta):
        phi = np.asarray(phi, dtype=np.float64)
        theta = np.asarray(theta, dtype=np.float64)
        x, s = np.cos(theta), np.sin(theta)
        out = np.zeros_like(phi)
        pmm = np.full_like(theta, np.sqrt(1 / (4 * np.pi)))
        for m in range(L_max + 1):
            if m > 0:
                pmm = -pmm * np.sqrt((2 * m + 1) / (2 * m)) * s
            p_prev, p = None, pmm
            cm, sm = np.cos(m * phi), np.sin(m * phi)
            for l in range(m, L_max + 1):
                if l == m + 1:
                    p_prev, p = p, np.sqrt(2 * m + 3) * x * pmm
                elif l > m + 1:
                    al = np.sqrt((4 * l * l - 1) / (l * l - m * m))
                    bl = np.sqrt(((l - 1) ** 2 - m * m) / (4 * (l - 1) ** 2 - 1))
                    p_prev, p = p, al * (x * p - bl * p_prev)
                if l == 0:
                    continue
                if m == 0:
                    out += a[l, l] * p
                else:
                    out += np.sqrt(2) * p * (a[l, l + m] * cm + a[l, l - m] * sm)
        return out
    return omega, a
