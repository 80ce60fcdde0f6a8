"""Host-side set-up: Julia range semantics and the slump/collapse geometry.

Point and node counts are those the reference's own set-up code produces
(utils/setup/mpts/get_slump.jl, mpts_populate.jl, mesh/get_coords.jl); the
known-answer cases of Julia's float ranges are documented Base behaviour.
"""
import numpy as np
import pytest

from epgpu import config, ic_collapse, ic_slump
from epgpu.julia import frange, rat


def test_julia_ranges_known_answers():
    # the documented motivation of Julia's twice-precision ranges
    assert frange(0.1, 0.1, 0.3) == [0.1, 0.2, 0.3]
    r = frange(0.0, 0.1, 1.0)
    assert len(r) == 11 and r[-1] == 1.0 and r[3] == 0.3
    # naive repeated stepping would give 0.30000000000000004
    assert 0.1 + 2 * 0.1 != 0.3
    assert frange(0.0, 1.0, 10.0) == [float(k) for k in range(11)]
    assert frange(1.0, 1.0, 0.0) == []
    assert rat(1.60396) == (40099, 25000)


def test_julia_range_fallback_branch():
    # an endpoint without a small rational: elements are start + (i-1)*step
    t0 = 10.000000000000002
    r = frange(t0, 1.0, 15.0)
    assert r[0] == t0 and all(r[i] == t0 + i * 1.0 for i in range(len(r)))


def test_slump_config1_geometry():
    ic, cfg = ic_slump([64.1584, 64.1584 / 4.0], [40, 10])
    m, p = ic["mesh"], ic["mpts"]
    assert p.nmp == 591
    assert m.nnodes == 451 and m.nel == [40, 10, 400] and m.nno == [41, 11, 451]
    assert m.h[0] == 64.1584 / 40 and m.h[1] == 16.0396 / 10
    # coordinates are the correctly rounded decimals k*h (Julia range), not k*fl(h)
    assert m.axes[0][-1] == 64.1584 and m.axes[1][-1] == 16.0396
    # roller boundaries on all four sides (require.jl:51-56)
    assert m.bcs[0].sum() == 2 * 11 and m.bcs[1].sum() == 2 * 41
    # friction: residual angle in the base layer z <= 2 wl = 3.84 m (get_slump.jl:91-92)
    assert np.all(p.phi[p.x[1] <= 3.84] == 7.5 * np.pi / 180)
    assert np.all(p.phi[p.x[1] > 3.84] == 20.0 * np.pi / 180)
    assert np.all(p.Omega0 == (m.h[0] / 2) * (m.h[1] / 2))
    # every B-spline node class is valid (no "Invalid position" on this mesh)
    from epgpu.abi import MeshView  # noqa: F401 (import check)


def test_slump_config2_geometry():
    ic, _ = ic_slump([64.1584, 16.0396], [640, 160], ni=3)
    assert ic["mpts"].nmp == 365024 and ic["mesh"].nnodes == 103201


def test_e2n_layout():
    ic, _ = ic_slump([64.1584, 64.1584 / 4.0], [40, 10])
    e2n = ic["mesh"].e2n
    # element 1 (x index 1, z index 1): the -1 row/column is outside -> 0
    assert e2n[:, 0].tolist()[:5] == [0, 0, 0, 0, 0]
    assert e2n[5, 0] == 1 and e2n[6, 0] == 2 and e2n[9, 0] == 1 + 11
    assert e2n.max() == 451 and e2n.shape == (16, 400)


def test_collapse_geometry():
    ic, _ = ic_collapse([5, 10], 0.0, 1.0e4, 80.0, 50.0)
    assert ic["mpts"].nmp == 160 and ic["time"]["te"] == 358.0


def test_kwargser_top_level_merge():
    instr = config.kwargser({"fwrk": {"deform": "infinitesimal", "trsfr": "std", "C_pf": 1.0, "musl": True,
                                      "locking": False, "damping": 0.1}})
    assert instr["fwrk"]["deform"] == "infinitesimal" and instr["basis"]["which"] == "bsmpm"
    # a partial group drops the other keys of that group, as in the reference
    with pytest.raises(config.UnsupportedError):
        config.kwargser({"fwrk": {"deform": "finite", "trsfr": "std"}})
    fw = {"deform": "finite", "trsfr": "apic", "C_pf": 1.0, "musl": True, "locking": True, "damping": 0.1}
    assert config.to_abi(config.kwargser({"fwrk": fw}))["trsfr"] == 2          # EP_TRSFR_APIC
    with pytest.raises(config.UnsupportedError):                               # mapsto.jl:44
        config.kwargser({"fwrk": {**fw, "trsfr": "flip"}})
    with pytest.raises(config.UnsupportedError):
        config.kwargser({"basis": {"which": "gimpm", "how": None, "ghost": True}})
    with pytest.warns(UserWarning):
        config.kwargser({"nonsense": 1})


def test_ensemble_rejects_meshes_whose_bspline_classes_break_the_partition_of_unity():
    """nel = [320, 80]: the node at xB - h along x is 7e-15 off the rounded xB - h, so the reference's
    exact comparison (bsmpm.jl:63-76) gives it the interior piece; the weights near that boundary then
    sum to 1.16 instead of 1 (the restatement oracle/pointmath.py shows it) and the slump moves without
    load.  The ensemble's mesh check counts that node; nel = [319, 79] is sound."""
    import pointmath as pm
    from epgpu.batch import bspline_invalid_nodes
    for nx, broken in ((320, True), (319, False), (40, False)):
        ic, _ = ic_slump([64.1584, 16.0396], [nx, nx // 4], ni=2)
        m = ic["mesh"]
        xn = np.unique(m.x[0])
        x0, x1, h = float(m.xB[0, 0]), float(m.xB[0, 1]), float(m.h[0])
        xp = np.linspace(x0, x1, 4001)[1:-1]
        e = np.clip(np.floor((xp - x0) / h), 0, xn.size - 2).astype(int)
        tot = np.zeros_like(xp)
        for o in (-1, 0, 1, 2):
            j = e + o
            ok = (j >= 0) & (j < xn.size)
            j = np.clip(j, 0, xn.size - 1)
            w, _ = pm.bspline((xp - xn[j]) / h, xn[j], x0, x1, h)
            tot += np.where(ok, w, 0.0)
        assert (np.abs(tot - 1.0).max() > 0.1) == broken, nx
        assert (bspline_invalid_nodes(m) > 0) == broken, nx
