"""FP64 conservation sums on the device (epgpu_conservation) against the same sums formed on the host
from the oracle's state with exactly rounded summation (math.fsum).

Bounds: the FP64 step's state equals the oracle's bit for bit, so its sums differ only by the order of
the FP64 additions: 1e-12 relative (mass, energies; momenta relative to Σ|ρΩ v|).  The mixed steps'
sums follow their state: the point mass ρ0Ω0 to FP32 rounding and the FP32 nodal masses to 1e-6, kinetic
and elastic energy to the mixed-precision stress bound 1e-5.  Two calls on the same state give the same bits (fixed-order
reductions).  In finite strain the nodal sums check the transfers themselves: Σ m_n = Σ ρΩ (partition
of unity, p2n.jl:71-75) and, with mUSL, Σ p_n = Σ ρΩ v (augm.jl:13-25).
"""
import copy
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

C1 = ([64.1584, 64.1584 / 4.0], [40, 10])
C1_3D = ([64.1584, 16.0396, 16.0396], [16, 4, 4])


def host_sums(m, mesh, finite, Del):
    """The sums of epgpu_conservation from a downloaded state, exactly rounded (math.fsum)."""
    ms = np.asarray(m.rho) * np.asarray(m.Omega)
    v = np.asarray(m.v)
    st = np.asarray(m.tau if finite else m.sig)
    x = np.linalg.solve(Del, st)
    w = 0.5 * np.einsum("kp,kp->p", st, x) * np.asarray(m.Omega0 if finite else m.Omega)
    return {"mass": math.fsum(ms), "momentum": np.array([math.fsum(ms * v[d]) for d in range(v.shape[0])]),
            "kinetic": math.fsum(0.5 * ms * (v * v).sum(axis=0)), "elastic": math.fsum(w),
            "mass_nodes": math.fsum(np.asarray(mesh.mi).ravel()),
            "momentum_nodes": np.array([math.fsum(np.asarray(mesh.p)[d]) for d in range(v.shape[0])]),
            "momentum_scale": math.fsum(np.abs(ms * v).sum(axis=0))}


def _rel(a, b, scale=None):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / (scale if scale else max(np.max(np.abs(b)), 1e-300)))


def _compare(got, want, tol_mass, tol_energy, tol_mom):
    ms = want["momentum_scale"]
    errs = {"mass": _rel(got["mass"], want["mass"]), "mass_nodes": _rel(got["mass_nodes"], want["mass_nodes"]),
            "momentum": _rel(got["momentum"], want["momentum"], ms),
            "momentum_nodes": _rel(got["momentum_nodes"], want["momentum_nodes"], ms),
            "kinetic": _rel(got["kinetic"], want["kinetic"]), "elastic": _rel(got["elastic"], want["elastic"])}
    bad = {k: v for k, v in errs.items()
           if v > {"mass": tol_mass, "mass_nodes": tol_mass, "kinetic": tol_energy, "elastic": tol_energy}.get(k, tol_mom)}
    assert not bad, (bad, errs)
    return errs


@pytest.mark.parametrize("case", ["2d_finite", "2d_infinitesimal_tpic", "3d_finite"])
@pytest.mark.parametrize("precision", ["fp64", "mixed_df"])
def test_conservation_sums_match_the_oracle(oracle_mod, case, precision):
    from epgpu import Engine, ic_slump
    mesh_args = C1_3D if case.startswith("3d") else C1
    kw = {"nonloc": {"status": False, "ls": 0.5}}
    if "infinitesimal" in case:
        kw["fwrk"] = {"deform": "infinitesimal", "trsfr": "tpic", "C_pf": 0.99, "musl": True, "locking": True,
                      "damping": 0.1}
    ic, cfg = ic_slump(*mesh_args, **kw)
    finite = cfg["instr"]["fwrk"]["deform"] == "finite"
    instr = copy.deepcopy(cfg["instr"])
    if precision != "fp64":
        instr["gpu"] = {"precision": precision, "jaumann": False}
    o = oracle_mod.Oracle(copy.deepcopy(ic), cfg["instr"])
    e = Engine(copy.deepcopy(ic), instr)
    t = 0.0
    windows = ((0, 1.0), (1, 1.5)) if not case.startswith("3d") else ((0, 0.5), (1, 0.8))
    for phase, T in windows:
        to, _ = o.run(phase, T, 10.0, t)
        te, _ = e.run(phase, T, 10.0, t)
        assert to == te
        t = te
    Del = np.asarray(ic["cmpr"]["Del"], dtype=np.float64)
    Del = Del.reshape(int(round(np.sqrt(Del.size))), -1, order="F")
    want = host_sums(o.download(), o.download_mesh(), finite, Del)
    got = e.conservation()
    again = e.conservation()
    assert all(np.array_equal(np.asarray(got[k]), np.asarray(again[k])) for k in got)     # fixed order
    if precision == "fp64":
        errs = _compare(got, want, 1e-12, 1e-12, 1e-12)
    else:
        errs = _compare(got, want, 1e-6, 1e-5, 1e-5)       # FP32 nodal masses: Σ m_n to 1e-6
    print(f"conservation {case} {precision}: " + ", ".join(f"{k} {v:.1e}" for k, v in errs.items())
          + f"; mass {got['mass']:.6e} kinetic {got['kinetic']:.4e} elastic {got['elastic']:.4e}")
    # the transfers' own identities in finite strain, where ρΩ = ρ0Ω0 does not change within a step
    # (infinitesimal_deform updates Ω but not ρ, deform.jl:25-44): Σ m_n = Σ ρΩ and Σ p_n = Σ ρΩ v
    if finite:
        assert _rel(got["mass_nodes"], got["mass"]) < (1e-12 if precision == "fp64" else 1e-6)
        assert _rel(got["momentum_nodes"], got["momentum"], want["momentum_scale"]) < (
            1e-12 if precision == "fp64" else 1e-5)
    assert got["kinetic"] > 0 and got["elastic"] > 0
