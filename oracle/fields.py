"""Initial vorticity fields (oracle restatement of the barotropic fields of
cmm_s2/core/dynamical_fields.py:181-214) and the synthetic fields of the
benchmark configurations."""
import numpy as np

pi = np.pi


def rossby_wave(phi, theta, t=0.0):
    """Rossby-Haurwitz wave (l,m) = (5,4), exact travelling solution
    (dynamical_fields.py:205-210)."""
    ell = 5
    alpha = 1 / (ell * (ell + 1))
    Omega = 2 * pi
    return 30 * np.cos(theta) * np.cos(4 * (phi + 2 * Omega * alpha * t)) * np.sin(theta) ** 4


def perturbed_rossby_wave(phi, theta):
    """dynamical_fields.py:213-215."""
    return 30 * np.cos(theta) * np.cos(4 * phi) * np.sin(theta) ** 4 + 0.1 * np.sin(theta) * np.cos(30 * theta)


def zonal_jet(phi, theta):
    """dynamical_fields.py:181-186."""
    beta2 = 12 ** 2
    theta_c = pi / 4
    u_lt = (pi / 2) * np.exp(-2 * beta2 * (1 - np.cos(-theta + pi / 2 - theta_c)))
    return (np.cos(-theta + pi / 2) * (2 * beta2 * (np.cos(theta_c) * np.sin(-theta + pi / 2)
                                                    - np.sin(theta_c) * np.cos(-theta + pi / 2)))
            + np.sin(pi / 2 - theta)) * u_lt


def perturbed_zonal_jet(phi, theta):
    """dynamical_fields.py:188-192."""
    beta2 = 12 ** 2
    theta_c = pi / 4 + 0.01 * np.cos(12 * phi)
    u_lt = (pi / 2) * np.exp(-2 * beta2 * (1 - np.cos(-theta + pi / 2 - theta_c)))
    return (np.cos(-theta + pi / 2) * (2 * beta2 * (np.cos(theta_c) * np.sin(-theta + pi / 2)
                                                    - np.sin(theta_c) * np.cos(-theta + pi / 2)))
            + np.sin(pi / 2 - theta)) * u_lt


def multi_jet(phi, theta):
    """dynamical_fields.py:195-198."""
    return perturbed_zonal_jet(phi, theta) + perturbed_zonal_jet(phi, theta - pi / 8)


def gaussian_vortex(phi, theta):
    """dynamical_fields.py:200-203."""
    x, y, z = np.sin(theta) * np.cos(phi), np.sin(theta) * np.sin(phi), np.cos(theta)
    sigma, C = 1 / 16, 4 * pi
    return C * np.exp(-((x - 1) ** 2 + y ** 2 + z ** 2) / sigma)


def gaussian_zonal_jets(phi, theta, lats=(0.5, -0.5, 1.1, -1.1), width=0.1, amplitude=10.0):
    """Zonal Gaussian jets in latitude: sum_j A exp(-((pi/2 - theta - lat_j)/w)^2)."""
    lat = pi / 2 - theta
    out = np.zeros_like(np.asarray(theta, dtype=np.float64) + 0 * phi)
    for lj in lats:
        out = out + amplitude * np.exp(-((lat - lj) / width) ** 2)
    return out


def sh_series(coeffs):
    """Real orthonormal spherical-harmonic series with coefficients
    coeffs (lmax+1, 2 lmax+1), column l + m for -l <= m <= l:
    m = 0 -> Pbar_l0; m > 0 -> sqrt2 Pbar_lm cos(m phi); m < 0 ->
    sqrt2 Pbar_l|m| sin(|m| phi)."""
    lmax = coeffs.shape[0] - 1

    def f(phi, theta):
        phi = np.asarray(phi, dtype=np.float64)
        theta = np.asarray(theta, dtype=np.float64)
        x, s = np.cos(theta), np.sin(theta)
        out = np.zeros(np.broadcast(phi, theta).shape)
        pmm = np.full(theta.shape, np.sqrt(1 / (4 * pi)))
        for m in range(lmax + 1):
            if m > 0:
                pmm = -pmm * np.sqrt((2 * m + 1) / (2 * m)) * s
            p_prev, p = None, pmm
            for l in range(m, lmax + 1):
                if l == m + 1:
                    p_prev, p = p, np.sqrt(2 * m + 3) * x * pmm
                elif l > m + 1:
                    a = np.sqrt((4 * l * l - 1) / (l * l - m * m))
                    b = np.sqrt(((l - 1) ** 2 - m * m) / (4 * (l - 1) ** 2 - 1))
                    p_prev, p = p, a * (x * p - b * p_prev)
                if m == 0:
                    out = out + coeffs[l, l] * p
                else:
                    out = out + np.sqrt(2) * p * (coeffs[l, l + m] * np.cos(m * phi)
                                                  + coeffs[l, l - m] * np.sin(m * phi))
        return out
    return f
