"""The random-field generator on the CPU: the library's spectrum draws against the numpy
restatement (oracle/grf_oracle.py), and the covariance one realization carries."""
import math

import numpy as np
import pytest


@pytest.mark.parametrize("dim,cov", [(2, "exponential"), (3, "exponential"), (2, "gaussian"), (3, "gaussian")])
def test_spectrum_matches_restatement(dim, cov):
    from epgpu import grf
    import grf_oracle as go
    g = grf.make_grf(dim, cov, [5.0, 4.0, 3.0][:dim], nh=400, seed=77)
    k, ab = grf.spectrum(g)
    k2, ab2 = go.spectrum(dim, cov, [5.0, 4.0, 3.0], 400, 77)
    np.testing.assert_allclose(k, k2, rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(ab, ab2, rtol=1e-12, atol=1e-14)


@pytest.mark.parametrize("dim", [2, 3])
def test_one_realization_has_the_exponential_covariance(dim):
    # the field's own (spatially averaged) covariance at lag r is
    # std^2 / nh * sum_k (xi_k^2 + eta_k^2) / 2 cos(kappa_k . r); it approaches exp(-|r|/ell)
    import grf_oracle as go
    ell = 5.0
    k, ab = go.spectrum(dim, "exponential", [ell] * 3, 5000, 1234)
    w = 0.5 * (ab ** 2).sum(axis=1) / 5000
    for r in (0.0, 2.5, 5.0, 10.0):
        lag = np.zeros(dim)
        lag[0] = r
        c = float((w * np.cos(k @ lag)).sum())
        assert abs(c - math.exp(-r / ell)) < 0.06, (r, c)


def test_gaussian_covariance_realization():
    import grf_oracle as go
    k, ab = go.spectrum(2, "gaussian", [2.5, 2.5], 5000, 9)
    w = 0.5 * (ab ** 2).sum(axis=1) / 5000
    for r in (0.0, 1.25, 2.5, 5.0):
        c = float((w * np.cos(k[:, 0] * r)).sum())
        assert abs(c - math.exp(-(r / 2.5) ** 2)) < 0.06, (r, c)


def test_grf_arguments_are_checked_without_gpu():
    import ctypes as C
    from epgpu import abi, grf
    lib = abi.load_library()
    g = grf.make_grf(2, "exponential", [5.0, 5.0], nh=10)
    g.ell[1] = 0.0
    out = np.zeros(4)
    x = np.zeros(8)
    assert lib.epgpu_grf_points(C.byref(g), x.ctypes.data_as(C.POINTER(C.c_double)), 4,
                                out.ctypes.data_as(C.POINTER(C.c_double))) == 1
