"""Oracle (test infrastructure only): numpy restatement of the linear
transport test flows and tracer fields of cmm_s2/core/dynamical_fields.py
and of the smooth test function of cmm_s2/tests/test_spherical_transport.py,
with the reference's formulas and the module constants T = 1, alpha = 0
as defaults.  Points are (3, N) as the reference's ``X`` arrays; the
velocities plug into oracle.evolution's integrators as V(t, dt, X)."""
import numpy as np

pi = np.pi
RHO0 = 3.0  # dynamical_fields.py:44


def _rot_x(a):
    return np.array([[1, 0, 0], [0, np.cos(a), -np.sin(a)], [0, np.sin(a), np.cos(a)]])


def _rot_y(a):
    return np.array([[np.cos(a), 0, -np.sin(a)], [0, 1, 0], [np.sin(a), 0, np.cos(a)]])


def _rot_z(a):
    return np.array([[np.cos(a), -np.sin(a), 0], [np.sin(a), np.cos(a), 0], [0, 0, 1]])


def _rotate(L, X):
    return np.array([L[0, 0] * X[0] + L[0, 1] * X[1] + L[0, 2] * X[2],
                     L[1, 0] * X[0] + L[1, 1] * X[1] + L[1, 2] * X[2],
                     L[2, 0] * X[0] + L[2, 1] * X[1] + L[2, 2] * X[2]])


def _cross(a, b):
    return np.array([a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]])


def _cart2sphere(X):
    """utils.cart2sphere (utils.py:18-23)."""
    x, y, z = X[0], X[1], X[2]
    phi = (np.arctan2(y, x) + 2 * pi) % (2 * pi)
    theta = np.arctan2(np.sqrt(y ** 2 + x ** 2), z)
    return phi, theta


def omega_r(theta):
    """dynamical_fields.py:48-55."""
    theta = np.asarray(theta, dtype=np.float64)
    out = np.zeros_like(theta)
    nz = theta != 0.0
    c = np.sin(theta[nz])
    out[nz] = (2 * pi) * np.sqrt(3) * (3 / 2) * (1 / (RHO0 * c)) * np.tanh(RHO0 * c) * (1 / np.cosh(RHO0 * c)) ** 2
    return out


def make_flow(kind, T=1.0, alpha=0.0):
    """The velocity V(t, dt, X) of flow `kind` (the names of
    dynamical_fields.py): 'u_sbr' :18-22, 'u_deform' :24-30,
    'u_deform_rot' :32-42, 'u_static_vortex' :57-65, 'u_rotating_vortex'
    :67-76, 'equator_vortex' :78-83, 'u_div' :97-107."""

    def u_sbr(t, dt, X):
        c = -2 * pi / T
        return _cross(X, [c * np.sin(alpha), 0, c * np.cos(alpha)])

    def u_deform(t, dt, X):
        c1 = 2 * 2 * np.cos(pi * t / T)
        return _cross(X, [0 * X[0], c1 * X[1], 0 * X[2]])

    def u_deform_rot(t, dt, X):
        tau = 2 * pi * t
        Xr = _rotate(_rot_z(tau).T @ _rot_y(alpha), X)
        return _rotate(_rot_y(alpha).T @ _rot_z(tau), u_deform(t, dt, Xr)) + u_sbr(t, dt, X)

    def u_static_vortex(t, dt, X):
        _, theta = _cart2sphere(X)
        w = omega_r(theta)
        return np.array([-X[1] * w, X[0] * w, 0 * X[2]])

    def u_rotating_vortex(t, dt, X):
        tau = 2 * pi * t / T
        Xr = _rotate(_rot_x(pi / 2) @ _rot_z(tau).T, X)
        return _rotate(_rot_z(tau) @ _rot_x(pi / 2).T, u_static_vortex(t, dt, Xr)) + u_sbr(t, dt, X)

    def equator_vortex(t, dt, X):
        Xr = _rotate(_rot_x(pi / 2), X)
        return _rotate(_rot_x(pi / 2).T, u_static_vortex(t, dt, Xr))

    def u_div(t, dt, X):
        phi, theta = _cart2sphere(X)
        ct = np.cos(pi * t / T)
        u = -(np.sin(phi / 2) ** 2) * np.sin(2 * theta) * np.sin(theta) * ct
        v = (-1 / 2) * np.sin(phi) * (np.sin(theta) ** 3) * ct
        A = [np.cos(theta) * np.cos(phi) * v - np.sin(theta) * np.sin(phi) * u,
             np.cos(theta) * np.sin(phi) * v + np.sin(theta) * np.cos(phi) * u,
             -np.sin(theta) * v]
        x, y, z = X[0], X[1], X[2]
        return np.array([(1 - x ** 2) * A[0] + (-x * y) * A[1] + (-x * z) * A[2],
                         (-x * y) * A[0] + (1 - y ** 2) * A[1] + (-y * z) * A[2],
                         (-x * z) * A[0] + (-y * z) * A[1] + (1 - z ** 2) * A[2]])

    return dict(u_sbr=u_sbr, u_deform=u_deform, u_deform_rot=u_deform_rot, u_static_vortex=u_static_vortex,
                u_rotating_vortex=u_rotating_vortex, equator_vortex=equator_vortex, u_div=u_div)[kind]


FLOWS = ["u_sbr", "u_deform", "u_deform_rot", "u_static_vortex", "u_rotating_vortex", "equator_vortex", "u_div"]

# bell centres and radius (dynamical_fields.py:110-119)
_H0, _R = 1.0, 0.5
_C1 = (pi + pi / 6, pi / 2)
_C2 = (pi - pi / 6, pi / 2)


def _bell_r(phi, theta, c):
    with np.errstate(invalid="ignore"):
        return np.arccos(np.sin(c[1] - pi / 2) * np.sin(theta - pi / 2)
                         + np.cos(c[1] - pi / 2) * np.cos(theta - pi / 2) * np.cos(phi - c[0]))


def cosine_bell(phi, theta):
    """dynamical_fields.py:122-137."""
    out = np.zeros_like(theta)
    for c in (_C1, _C2):
        r = _bell_r(phi, theta, c)
        with np.errstate(invalid="ignore"):
            m = r < _R
        out[m] += (_H0 / 2) * (1 + np.cos(r[m] * pi / _R))
    return 0.9 * out + 0.1


def slotted_cylinders(phi, theta):
    """IC_SC, dynamical_fields.py:139-157."""
    r1, r2 = _bell_r(phi, theta, _C1), _bell_r(phi, theta, _C2)
    o1, o2 = np.zeros_like(theta), np.zeros_like(theta)
    with np.errstate(invalid="ignore"):
        o1[(r1 <= _R) & (np.abs(phi - _C1[0]) >= _R / 6)] = 0.9
        o1[(r1 <= _R) & (np.abs(phi - _C1[0]) < _R / 6) & (theta < (-5 * _R / 12 + pi / 2))] = 0.9
        o2[(r2 <= _R) & (np.abs(phi - _C2[0]) >= _R / 6)] = 0.9
        o2[(r2 <= _R) & (np.abs(phi - _C2[0]) < _R / 6) & (theta > (5 * _R / 12 + pi / 2))] = 0.9
    return o1 + o2 + 0.1


def static_vort_ic(t, xyz):
    """dynamical_fields.py:85-88; xyz (3, N)."""
    phi, theta = _cart2sphere(xyz)
    rho = RHO0 * np.sin(theta)
    return 1 - np.tanh((rho / 5) * np.sin(phi - omega_r(theta) * t))


def rotating_vort_ic(t, xyz):
    """dynamical_fields.py:90-95."""
    return static_vort_ic(t, _rotate(_rot_x(pi / 2) @ _rot_z(0).T, xyz))


def smooth_test(xyz):
    """test_func of tests/test_spherical_transport.py:36-38; xyz (N, 3)."""
    x, y, z = xyz[:, 0], xyz[:, 1], xyz[:, 2]
    return np.sin(x ** 2) * (10 * np.cos(y - 2)) + np.cos(10 * z ** 5) + 2 * np.sin(x * 3 * (z - 0.1) + y ** 7)


def random_initial_condition(xyz):
    """dynamical_fields.py:158-172; xyz (3, N).  The module-level draws
    (np.random.seed(42); uniform(-1, 1, 33**2)) taken from a private
    RandomState with the same seed, so the global generator is untouched;
    scipy's sph_harm(m, l, phi, theta) is sph_harm_y(l, m, theta, phi)."""
    from scipy.special import sph_harm_y
    coeffs = np.random.RandomState(42).uniform(-1, 1, 33 ** 2)
    phi, theta = _cart2sphere(xyz)
    out, lm = 0, 0
    for l in range(33):
        for m in range(-l, l):
            out = out + coeffs[lm] * sph_harm_y(l, m, theta, phi).real
            lm += 1
    return out


def tracer(kind, X, t=0.0):
    """Tracer `kind` at points X (N, 3)."""
    if kind == "smooth_test":
        return smooth_test(X)
    if kind == "random_initial_condition":
        return random_initial_condition(X.T)
    if kind == "static_vort_IC":
        return static_vort_ic(t, X.T)
    if kind == "rotating_vort_IC":
        return rotating_vort_ic(t, X.T)
    phi, theta = _cart2sphere(X.T)
    return {"cosine_bell": cosine_bell, "IC_SC": slotted_cylinders}[kind](phi, theta)


TRACERS = ["cosine_bell", "IC_SC", "static_vort_IC", "rotating_vort_IC", "smooth_test",
           "random_initial_condition"]
