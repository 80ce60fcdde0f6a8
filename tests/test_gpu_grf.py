"""The random field on the GPU against the FP64 restatement, and the c2 slump's cohesion."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dim,cov", [(2, "exponential"), (3, "exponential"), (2, "gaussian")])
def test_field_matches_restatement(dim, cov):
    from epgpu import grf
    import grf_oracle as go
    rng = np.random.default_rng(dim)
    X = rng.uniform(0.0, 64.0, (20_000, dim))
    g = grf.make_grf(dim, cov, [5.0, 4.0, 3.0][:dim], mean=2e4, std=6e3, vmin=-1e30, nh=5000, seed=31)
    f = grf.points(g, X)
    ref = go.field(X, dim, cov, [5.0, 4.0, 3.0], 2e4, 6e3, -1e30, 5000, 31)
    err = np.abs(f - ref).max() / 6e3
    print(f"{dim}d {cov}: max |gpu - fp64| / std = {err:.2e}")
    assert err < 1e-4


def test_slump_cohesion_field():
    from epgpu import ic_slump
    ic, cfg = ic_slump([64.1584, 16.0396], [640, 160], ni=3,
                       grf={"status": True, "covariance": "exponential",
                            "param": {"Ix": [5.0, 5.0], "mean": 2.0e4, "cov": 0.3, "min": 1.0e3, "seed": 1234}},
                       nonloc={"status": False, "ls": 0.5})
    c0 = ic["mpts"].c0
    print(f"c2 cohesion: mean {c0.mean():.4e}, std {c0.std():.4e}, min {c0.min():.4e}, n {c0.size}")
    assert c0.size == 365_024 and c0.min() >= 1e3
    assert abs(c0.mean() - 2e4) < 0.25 * 2e4 and 0.4 * 6e3 < c0.std() < 1.6 * 6e3
