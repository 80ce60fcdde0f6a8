"""The mixed-precision 3d step (infinitesimal strain) against the FP64 oracle: the config-3
switches (GIMP / TPIC / J2), the B-spline basis, DP and standard USL with mUSL and F-bar."""
import copy

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

C1_3D = ([64.1584, 16.0396, 16.0396], [16, 4, 4])
STRESS_TOL = 1e-5
DISP_TOL = 1e-4

J2 = {"plast": {"status": True, "constitutive": "J2"}}
C3_FWRK = {"deform": "infinitesimal", "trsfr": "tpic", "C_pf": 0.0, "musl": False, "locking": False, "damping": 0.1}
# (switches, material overrides, shift of the points in units of h).  GIMP cases shift the lattice
# by 1e-3 h: the reference's lattice puts points on GIMP support edges (l = h/4), where a node
# gets a mass ~ r^2 and a force ~ r (r: distance to the edge), an acceleration ~ 1/r; there the
# FP64 result depends on 1e-15-level rounding of r (ghost padding shifts node coordinates by an
# ulp) that FP32 offsets (~1e-7 h) cannot resolve.  Unshifted, config 3 differs by 1e-1 in stress;
# shifted by 1e-3 h it agrees to 4e-6 (see test_gimp_support_edges below).
CASES = {
    "config3": (dict(basis={"which": "gimpm", "how": "undeformed", "ghost": True}, fwrk=C3_FWRK, **J2),
                {"c0": 5.0e4, "Hp": 1.0e5}, 1e-3),
    "config3_bsmpm": (dict(fwrk=C3_FWRK, **J2), {"c0": 5.0e4, "Hp": 1.0e5}, 0.0),
    "config3_gimp_noghost": (dict(basis={"which": "gimpm", "how": "undeformed", "ghost": False}, fwrk=C3_FWRK, **J2),
                             {"c0": 5.0e4, "Hp": 1.0e5}, 1e-3),
    "bsmpm_dp_musl_fbar": ({"fwrk": {"deform": "infinitesimal", "trsfr": "std", "C_pf": 1.0, "musl": True,
                                     "locking": True, "damping": 0.1}}, None, 0.0),
    "bsmpm_j2_fbar_tpic": (dict(fwrk={"deform": "infinitesimal", "trsfr": "tpic", "C_pf": 0.5, "musl": True,
                                      "locking": True, "damping": 0.1}, **J2), {"c0": 5.0e4, "Hp": 1.0e5}, 0.0),
    "gimp_j2_fbar_tpic": (dict(basis={"which": "gimpm", "how": "undeformed", "ghost": False},
                               fwrk={"deform": "infinitesimal", "trsfr": "tpic", "C_pf": 0.5, "musl": True,
                                     "locking": True, "damping": 0.1}, **J2), {"c0": 5.0e4, "Hp": 1.0e5}, 1e-3),
}


def _compare(oracle_mod, kw, over, shift, precision):
    from epgpu import Engine, ic_slump
    ic, cfg = ic_slump(*C1_3D, cmpr_over=over, nonloc={"status": False, "ls": 0.5}, **kw)
    if over:
        ic["mpts"].c0[:] = over["c0"]
    ic["mpts"].x += shift * ic["mesh"].h[0]
    x0 = ic["mpts"].x.copy()
    o = oracle_mod.Oracle(copy.deepcopy(ic), cfg["instr"])
    instr = copy.deepcopy(cfg["instr"])
    instr["gpu"] = {"precision": precision, "jaumann": False}
    e = Engine(copy.deepcopy(ic), instr)
    t = 0.0
    for phase, T in ((0, 0.3), (1, 0.5)):
        to, _ = o.run(phase, T, 10.0, t)
        te, _ = e.run(phase, T, 10.0, t)
        assert to == te
        t = te
    a, b = e.download(), o.download()
    s = float(np.linalg.norm(a.sig - b.sig) / np.linalg.norm(b.sig))
    d = float(np.linalg.norm(a.x - b.x) / max(np.linalg.norm(b.x - x0), 1e-300))
    return a, b, s, d


def test_gimp_support_edges(oracle_mod):
    # the unshifted config-3 lattice: reported, bounded loosely (the FP64 reference is rounding-driven there)
    kw, over, _ = CASES["config3"]
    _, _, s0, d0 = _compare(oracle_mod, kw, over, 0.0, "mixed")
    _, _, s1, d1 = _compare(oracle_mod, kw, over, 1e-3, "mixed")
    print(f"config3 GIMP lattice on support edges: stress {s0:.3e} displacement {d0:.3e}; "
          f"shifted 1e-3 h: stress {s1:.3e} displacement {d1:.3e}")
    assert s1 < STRESS_TOL and d1 < DISP_TOL
    assert np.isfinite(s0) and s0 < 0.5


@pytest.mark.parametrize("precision", ["mixed", "mixed_df"])
@pytest.mark.parametrize("case", list(CASES))
def test_mixed3d_vs_oracle(oracle_mod, case, precision):
    kw, over, shift = CASES[case]
    e_a, b, s, d = _compare(oracle_mod, kw, over, shift, precision)
    print(f"3d {case} {precision} (shift {shift} h): stress {s:.3e} displacement {d:.3e}")
    assert s < STRESS_TOL and d < DISP_TOL
    assert np.abs(e_a.Fij - b.Fij).max() < 1e-5


def test_mixed3d_finite_strain_is_reported_unsupported():
    from epgpu import Engine, ic_slump
    from epgpu.abi import EPError
    ic, cfg = ic_slump(*C1_3D, nonloc={"status": False, "ls": 0.5})
    instr = copy.deepcopy(cfg["instr"])
    instr["gpu"] = {"precision": "mixed", "jaumann": False}
    with pytest.raises(EPError) as ex:
        Engine(ic, instr)
    assert ex.value.status == 2
