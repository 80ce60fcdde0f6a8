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
