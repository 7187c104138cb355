"""The torch FP64 restatement of the composition (oracle.compose_torch),
the reference gradient of the composition adjoint, against the numpy
oracle: same composed points, and its autograd gradient equal to centred
differences of the oracle's own composition along random directions."""
import numpy as np
import torch

from oracle import geometry as G
from oracle import spline as SP
from oracle.compose_torch import composite_eval


def _setup(n_q=400):
    from cmm_gpu import meshgen, workloads
    verts, tris = meshgen.icosahedral_mesh(3)
    tan, s_pts = meshgen.stencil_frames(verts)
    jets = workloads.submap_stack(s_pts, tan, 3, seed=2)
    loc = G.ConeLocator(verts, tris)
    comp = SP.CompositeOracle(verts, tris, loc, jets, closed=True)
    q = meshgen.random_sphere_points(n_q, seed=4)
    return verts, tris, loc, comp, q


def test_restatement_matches_oracle_composition():
    verts, tris, loc, comp, q = _setup()
    cs = [torch.from_numpy(c) for c in comp.coeffs]
    out = composite_eval(cs, torch.from_numpy(q), verts, tris, loc).numpy()
    assert np.abs(out - comp(q)).max() < 1e-14


def test_restatement_gradient_matches_oracle_differences():
    verts, tris, loc, comp, q = _setup()
    rng = np.random.default_rng(7)
    y = rng.standard_normal(q.shape)
    cs = [torch.from_numpy(c.copy()).requires_grad_(True) for c in comp.coeffs]
    qt = torch.from_numpy(q.copy()).requires_grad_(True)
    (composite_eval(cs, qt, verts, tris, loc) * torch.from_numpy(y)).sum().backward()
    base = comp.coeffs.copy()
    h = 1e-6

    def J(coeffs, pts):
        comp.coeffs = coeffs
        return float((comp(pts) * y).sum())

    for k in range(len(cs)):
        d = rng.standard_normal(base[k].shape)
        cp, cm = base.copy(), base.copy()
        cp[k] += h * d
        cm[k] -= h * d
        fd = (J(cp, q) - J(cm, q)) / (2 * h)
        ad = float((cs[k].grad.numpy() * d).sum())
        assert abs(fd - ad) < 1e-8 * abs(ad), (k, fd, ad)
    dq = rng.standard_normal(q.shape)
    dq -= (dq * q).sum(1, keepdims=True) * q
    fd = (J(base, q + h * dq) - J(base, q - h * dq)) / (2 * h)
    ad = float((qt.grad.numpy() * dq).sum())
    assert abs(fd - ad) < 1e-8 * abs(ad), (fd, ad)
    # the composition is invariant to scaling q, so its gradient is tangent
    assert np.abs((qt.grad.numpy() * q).sum(1)).max() < 1e-10 * np.abs(qt.grad.numpy()).max()


def test_vorticity_restatement_matches_oracle_series():
    """oracle.vorticity_torch against oracle.fields.sh_series: values, and
    the autograd point gradient against centred differences of the numpy
    series along tangent directions."""
    from cmm_gpu import meshgen, workloads
    from oracle import fields as F
    from oracle.vorticity_torch import sh_series_at
    _, a = workloads.random_sh_vorticity(6, seed=1)
    X = meshgen.random_sphere_points(500, seed=2)

    def series(P):
        P = P / np.linalg.norm(P, axis=1, keepdims=True)
        return F.sh_series(a)(np.arctan2(P[:, 1], P[:, 0]), np.arccos(np.clip(P[:, 2], -1, 1)))
    Xt = torch.from_numpy(X.copy()).requires_grad_(True)
    w = sh_series_at(torch.from_numpy(a), Xt)
    assert np.abs(w.detach().numpy() - series(X)).max() < 1e-12 * np.abs(series(X)).max()
    y = np.random.default_rng(3).standard_normal(len(X))
    (w * torch.from_numpy(y)).sum().backward()
    dX = np.random.default_rng(4).standard_normal(X.shape)
    dX -= (dX * X).sum(1, keepdims=True) * X
    h = 1e-6
    fd = float(((series(X + h * dX) - series(X - h * dX)) * y).sum()) / (2 * h)
    ad = float((Xt.grad.numpy() * dX).sum())
    assert abs(fd - ad) < 1e-8 * abs(ad), (fd, ad)


def _bve_case():
    from cmm_gpu import meshgen, workloads
    from oracle.bve_torch import BVETorch
    verts, tris = meshgen.icosahedral_mesh(3)
    _, a = workloads.random_sh_vorticity(6, seed=1)
    return verts, tris, a, BVETorch(verts, tris, 8, 10, 0.05, n_maps=4)


def test_whole_run_restatement_matches_oracle_run():
    """The torch restatement of the whole barotropic run (oracle.bve_torch,
    level 3, L = 8, 10 steps, remap every 4) against the numpy oracle's run
    with the same closed-form choices.  The map update's stencil
    differences over 4 eps = 4e-5 amplify rounding 2.5e4 times per step, so
    two FP64 evaluations of the same run agree to ~1e-11, not 1e-16."""
    from oracle.bve import BVEOracle
    from oracle import fields as OF
    verts, tris, a, bt = _bve_case()
    om = bt.omega_T(torch.from_numpy(a)).numpy()
    orc = BVEOracle(verts, tris, G.ConeLocator(verts, tris), 8, 10, 0.05, OF.sh_series(a), n_maps=4,
                    closed=True, tie_fix=True).run()
    assert np.abs(om - orc.last_omega).max() < 1e-10 * np.abs(orc.last_omega).max()


def test_whole_run_restatement_gradient_against_differences():
    """Its autograd gradient of J along a random direction against centred
    differences of its own J (h = 1e-5)."""
    verts, tris, a, bt = _bve_case()
    target = 0.9 * bt.omega_T(torch.from_numpy(a)).detach()
    J, g = bt.gradient(a, target)
    d = np.random.default_rng(3).standard_normal(a.shape)
    d[np.arange(7)[:, None] < np.abs(np.arange(13)[None, :] - np.arange(7)[:, None])] = 0   # |m| <= l only
    h = 1e-5

    def Jat(x):
        with torch.no_grad():
            return float((bt.W * (bt.omega_T(torch.from_numpy(x)) - target) ** 2).sum())

    fd = (Jat(a + h * d) - Jat(a - h * d)) / (2 * h)
    ad = float((g * d).sum())
    assert abs(fd - ad) < 1e-6 * abs(ad), (fd, ad)
