"""The learned return map on the CPU: the restated labels and network (oracle/mlp_oracle.py)
against finite differences, the shear-region closed form, and the library's own
host-side labels (include/epgpu.h epgpu_mlp_label)."""
import numpy as np
import pytest

L2G = 0.3 / (1.0 - 2.0 * 0.3)      # lambda / (2G) = nu / (1 - 2 nu) for nu = 0.3


def test_oracle_gradient_matches_finite_differences():
    import mlp_oracle as mo
    rng = np.random.default_rng(3)
    p = mo.init_params(1) * 0.5
    x = rng.normal(0.0, 1.0, (16, mo.NX)).astype(np.float32)
    t = rng.normal(0.0, 1.0, (16, mo.NY)).astype(np.float32)
    _, g = mo.loss_and_grad(p.astype(np.float64), x, t, bf=False)
    idx = rng.choice(mo.NPARAM, 40, replace=False)
    idx = np.concatenate([idx, [0, 767, 768, mo.NPARAM - 1, mo.NPARAM - 4, 50432]])   # W1, b1, W5, b5 ends
    h = 1e-6
    for i in idx:
        pp, pm = p.astype(np.float64).copy(), p.astype(np.float64).copy()
        pp[i] += h
        pm[i] -= h
        lp, _ = mo.loss_and_grad(pp, x, t, bf=False)
        lm, _ = mo.loss_and_grad(pm, x, t, bf=False)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 + 1e-4 * abs(fd), (i, fd, g[i])


def test_bf16_rounding_is_round_to_nearest_even():
    import mlp_oracle as mo
    a = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, -2.5, 3.14159265], dtype=np.float32)
    r = mo.bf16(a)
    assert r[0] == 1.0 and r[1] == 1.0                     # tie to even
    assert r[2] == np.float32(1.0 + 2 ** -7)
    assert r[3] == -2.5
    assert abs(r[4] - 3.140625) < 1e-7


def test_shear_region_label_is_the_unit_correction():
    # a shear return keeps P and scales the deviator: the correction per unit overstress is (-1, 1)
    import mlp_oracle as mo
    x = mo.sample_trials(2000, L2G, seed=5, spread=0.3)
    y, ok = mo.label(x, L2G)
    t1, t2 = mo.trial_stress(x[:, 0].astype(float), x[:, 1].astype(float), L2G)
    eta, xi = mo._dp_params(x[:, 4].astype(float))
    shear = ok & (0.5 * (t1 + t2) < xi / eta)
    assert shear.sum() > 1500
    np.testing.assert_allclose(y[shear, 0], -1.0, atol=2e-4)
    np.testing.assert_allclose(y[shear, 1], 1.0, atol=2e-4)


def test_labels_match_the_library_host_code():
    from epgpu import mlp
    import mlp_oracle as mo
    x = mo.sample_trials(3000, L2G, seed=11, spread=2.0)
    # add tension-side rows (the apex branch of DP.jl:53-58) and elastic rows
    rng = np.random.default_rng(2)
    xa = x[:500].copy()
    xa[:, 0] = rng.uniform(0.5, 4.0, 500)
    xa[:, 1] = xa[:, 0] - rng.uniform(0.0, 0.5, 500)
    xe = x[:200].copy()
    xe[:, 0], xe[:, 1] = -1.0, -1.01
    X = np.concatenate([x, xa, xe]).astype(np.float32)
    y_ref, ok = mo.label(X, L2G)
    y_lib = mlp.label(X, L2G)
    assert ok[:3000].all() and not ok[-200:].any()
    np.testing.assert_allclose(y_lib, y_ref, rtol=1e-5, atol=1e-5)


def test_features_restatement_scaling():
    # features of a trial strain carry the overstress the exact map sees
    import mlp_oracle as mo
    G, coh, tphi = 3.85e5, 1.5e4, np.tan(np.radians(20.0))
    e11, e22, e12 = np.array([-0.02]), np.array([-0.05]), np.array([0.01])
    x = mo.features(e11, e22, e12, coh, tphi, G, L2G)
    s = coh / (2 * G)
    em, r = 0.5 * (e11 + e22), np.hypot(0.5 * (e11 - e22), e12)
    np.testing.assert_allclose(x[0, :2], [(em + r)[0] / s, (em - r)[0] / s])
    # physical overstress from the Voigt stress = c * phi_n
    lam, mu = 2 * G * L2G, G
    sxx = lam * (e11 + e22) + 2 * mu * e11
    syy = lam * (e11 + e22) + 2 * mu * e22
    sxy = 2 * mu * e12
    P = 0.5 * (sxx + syy)
    tII = np.sqrt(0.25 * (sxx - syy) ** 2 + sxy ** 2)
    den = np.sqrt(9 + 12 * tphi ** 2)
    fs = tII + 3 * tphi / den * P - 3 * coh / den
    assert abs(max(fs[0], 0.0) / coh - x[0, 6]) < 1e-9


@pytest.mark.parametrize("n", [1, 130])
def test_forward_shapes_and_bf16_path(n):
    import mlp_oracle as mo
    p = mo.init_params(0)
    x = mo.sample_trials(n, L2G, seed=1)
    y, (H, Z) = mo.forward(p, x)
    assert y.shape == (n, mo.NOUT) and len(H) == 5 and len(Z) == 4
    y64, _ = mo.forward(p.astype(np.float64), x, bf=False)
    assert np.abs(y - y64).max() < 0.05 * max(np.abs(y64).max(), 1.0)


def _dp3_voigt(s, tphi):
    """The 3d DP return on a Voigt stress (xx, yy, zz, yz, xz, xy) as DP.jl:69-98 forms it (c = 1,
    psi = 0, outer cone DP.jl:19-21): the tensor form the principal-frame labels stand in for."""
    sphi, cphi = tphi / np.sqrt(1 + tphi ** 2), 1 / np.sqrt(1 + tphi ** 2)
    P = s[:, :3].mean(axis=1)
    t = s.copy()
    t[:, :3] -= P[:, None]
    tII = np.sqrt(0.5 * (t[:, :3] ** 2).sum(axis=1) + (t[:, 3:] ** 2).sum(axis=1))
    eta = 6 * sphi / (np.sqrt(3) * (3 + sphi))
    xi = 6 * cphi / (np.sqrt(3) * (3 + sphi))
    sm = xi / eta
    fs = tII + eta * P - xi
    hh = tII - (xi - eta * sm) - np.sqrt(1 + eta ** 2) * (P - sm)
    out = s.copy()
    shear = ((fs > 0) & (P < sm)) | ((hh > 0) & (P >= sm))
    r = (xi - eta * P) / tII
    out[shear] = t[shear] * r[shear, None]
    out[shear, :3] += P[shear, None]
    apex = (hh <= 0) & (P >= sm)
    out[apex] = 0.0
    out[apex, :3] = (sm - P)[apex, None]
    return out


def test_3d_labels_are_the_tensor_return_in_the_principal_frame():
    """A 3d label applied in a rotated frame equals the Voigt-form return of the rotated trial
    stress: the return is coaxial with the trial (isotropic stiffness), which the step relies on."""
    import mlp_oracle as mo
    x = mo.sample_trials(2000, L2G, seed=31, spread=1.0, dim=3)
    y, ok = mo.label(x, L2G)
    assert ok.all() and np.all(x[:, 7] == 1.0)
    e = x[:, :3].astype(np.float64)
    t = mo.trial_stress3(e, L2G)
    em, q, rr = mo.frame3(e)
    c = y[:, 0:1] * em + y[:, 1:2] * q + y[:, 2:3] * rr
    tr_ret = mo.trial_stress3(e + x[:, 6:7].astype(np.float64) * c, L2G)
    rng = np.random.default_rng(3)
    Q, _ = np.linalg.qr(rng.normal(size=(len(x), 3, 3)))
    T = np.einsum("nik,nk,njk->nij", Q, t, Q)
    voigt = np.stack([T[:, 0, 0], T[:, 1, 1], T[:, 2, 2], T[:, 1, 2], T[:, 0, 2], T[:, 0, 1]], axis=1)
    ret = _dp3_voigt(voigt, x[:, 4].astype(np.float64))
    R = np.einsum("nik,nk,njk->nij", Q, tr_ret, Q)
    rv = np.stack([R[:, 0, 0], R[:, 1, 1], R[:, 2, 2], R[:, 1, 2], R[:, 0, 2], R[:, 0, 1]], axis=1)
    # labels are float32: the returned stress is good to ~1e-6 of the overstress scale
    np.testing.assert_allclose(rv, ret, atol=2e-5 * np.abs(ret).max())
    # shear returns shrink the deviator radially (psi = 0): (0, -sqrt2, 0) in the trial's frame
    P = t.mean(axis=1)
    eta, xi = mo._dp_params3(x[:, 4].astype(np.float64))
    shear = P < xi / eta
    assert shear.sum() > 1500
    np.testing.assert_allclose(y[shear, :3], np.tile([0.0, -np.sqrt(2.0), 0.0], (int(shear.sum()), 1)), atol=2e-5)
    assert np.abs(mo.overstress3(tr_ret, x[:, 4].astype(np.float64))).max() < 1e-5


def test_3d_labels_match_the_library_host_code():
    from epgpu import mlp
    import mlp_oracle as mo
    x = mo.sample_trials(3000, L2G, seed=12, spread=2.0, dim=3)
    rng = np.random.default_rng(4)
    xa = x[:500].copy()                       # tension side: the apex branch of DP.jl:89-94
    xa[:, 0] = rng.uniform(0.5, 4.0, 500)
    xa[:, 1] = xa[:, 0] - rng.uniform(0.0, 0.5, 500)
    xa[:, 2] = xa[:, 1] - rng.uniform(0.0, 0.5, 500)
    xe = x[:200].copy()                       # elastic rows
    xe[:, 0], xe[:, 1], xe[:, 2] = -1.0, -1.005, -1.01
    X = np.concatenate([x, xa, xe]).astype(np.float32)
    y_ref, ok = mo.label(X, L2G)
    y_lib = mlp.label(X, L2G)
    assert ok[:3000].all() and not ok[-200:].any() and ok[3000:3500].any()
    np.testing.assert_allclose(y_lib, y_ref, rtol=1e-5, atol=1e-5)
    # the 2d rows of a mixed batch keep their own map
    x2 = mo.sample_trials(100, L2G, seed=1)
    Xm = np.concatenate([X[:100], x2]).astype(np.float32)
    np.testing.assert_allclose(mlp.label(Xm, L2G), mo.label(Xm, L2G)[0], rtol=1e-5, atol=1e-5)


def test_3d_features_carry_the_physical_overstress():
    import mlp_oracle as mo
    G, coh, tphi = 3.85e6, 3.0e4, np.tan(np.radians(25.0))
    rng = np.random.default_rng(0)
    A = rng.normal(scale=0.01, size=(50, 3, 3))
    eps = 0.5 * (A + A.transpose(0, 2, 1))
    x = mo.features3(eps, coh, tphi, G, L2G)
    assert np.all(x[:, 0] >= x[:, 1]) and np.all(x[:, 1] >= x[:, 2]) and np.all(x[:, 7] == 1)
    lam = 2 * G * L2G
    tr = np.trace(eps, axis1=1, axis2=2)
    S = lam * tr[:, None, None] * np.eye(3) + 2 * G * eps
    P = np.trace(S, axis1=1, axis2=2) / 3
    dev = S - P[:, None, None] * np.eye(3)
    tII = np.sqrt(0.5 * (dev * dev).sum(axis=(1, 2)))
    sphi, cphi = np.sin(np.radians(25.0)), np.cos(np.radians(25.0))
    fs = tII + 6 * sphi / (np.sqrt(3) * (3 + sphi)) * P - 6 * coh * cphi / (np.sqrt(3) * (3 + sphi))
    np.testing.assert_allclose(x[:, 6], np.maximum(fs, 0) / coh, atol=1e-9)
