import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "elastoplasm.jl_gb300"), os.path.join(ROOT, "oracle"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and runs through libepgpu.so")


# fields of the point state compared between the GPU step and the oracle
POINT_FIELDS = ["x", "v", "l", "n", "Omega", "dJ", "J", "rho", "dlam", "epII", "sig", "tau",
                "dvij", "dFij", "Fij", "bij", "eij", "wij", "sJij", "vmax"]


def compare_points(a, b, rtol=0.0, fields=POINT_FIELDS):
    """Max relative difference per field (scaled by the field's max magnitude); asserts <= rtol."""
    worst = {}
    for f in fields:
        x, y = np.asarray(getattr(a, f)), np.asarray(getattr(b, f))
        assert x.shape == y.shape, f
        scale = max(np.abs(y).max(initial=0.0), 1e-300)
        d = np.abs(x - y).max(initial=0.0) / scale
        if not (np.isfinite(x).all() == np.isfinite(y).all()):
            d = np.inf
        worst[f] = float(d)
    bad = {k: v for k, v in worst.items() if not v <= rtol}
    assert not bad, f"fields beyond rtol={rtol}: {bad}"
    return worst


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build()
    return oracle
