"""The Mohr-Coulomb (MCRetMap.jl) and modified Cam-Clay (camC.zip: camC/camCmodRetMap.jl) return maps
on the GPU, against the FP64 oracle: the FP64 step to the drop-in's 1e-10 (per field, including ϵpV,
which the Cam-Clay return writes), the mixed precisions (FP64 islands for the iterations) to the
mixed-mode targets, 1e-5 in stress and 1e-4 in displacement."""
import copy

import numpy as np
import pytest

from conftest import POINT_FIELDS, compare_points

pytestmark = pytest.mark.gpu

C1 = ([64.1584, 64.1584 / 4.0], [40, 10])
C1_3D = ([64.1584, 64.1584 / 4.0, 64.1584 / 4.0], [40, 10, 4])
CASES = [("MC", "finite", 2), ("MC", "infinitesimal", 2), ("camC", "finite", 2), ("camC", "infinitesimal", 2),
         ("camC", "finite", 3), ("camC", "infinitesimal", 3)]


def _ic(cons, deform, dim):
    from epgpu import ic_slump
    fw = {"deform": deform, "trsfr": "std", "C_pf": 1.0, "musl": True, "locking": True, "damping": 0.1}
    L, nel = C1 if dim == 2 else C1_3D
    return ic_slump(L, nel, fwrk=fw, plast={"status": True, "constitutive": cons},
                    nonloc={"status": False, "ls": 0.5})


def _windows(o, e, T0, T1):
    t = 0.0
    for phase, T in ((0, T0), (1, T1)):
        to, no = o.run(phase, T, 10.0, t)
        te, ne = e.run(phase, T, 10.0, t)
        assert (to, no) == (te, ne), ((to, no), (te, ne))
        t = te
    return t


@pytest.mark.parametrize("cons,deform,dim", CASES)
def test_fp64_step_matches_the_oracle(oracle_mod, cons, deform, dim):
    from epgpu import Engine
    ic, cfg = _ic(cons, deform, dim)
    o = oracle_mod.Oracle(copy.deepcopy(ic), cfg["instr"])
    e = Engine(copy.deepcopy(ic), cfg["instr"])
    _windows(o, e, 1.0, 2.0 if dim == 2 else 1.5)
    a, b = e.download(), o.download()
    assert (b.epII[0] > 0).sum() > 20
    if cons == "camC":
        assert (b.epV != 0).sum() > 20
    worst = compare_points(a, b, 1e-10, fields=POINT_FIELDS + ["epV"])
    print(cons, deform, dim, "max rel diff", max(worst.values()))
    e.close()


@pytest.mark.parametrize("precision", ["mixed", "mixed_df"])
@pytest.mark.parametrize("cons,deform,dim", CASES)
def test_mixed_step_matches_the_oracle(oracle_mod, cons, deform, dim, precision):
    from epgpu import Engine
    ic, cfg = _ic(cons, deform, dim)
    x0 = ic["mpts"].x.copy()
    instr = copy.deepcopy(cfg["instr"])
    instr["gpu"] = {"precision": precision, "jaumann": False}
    o = oracle_mod.Oracle(copy.deepcopy(ic), cfg["instr"])
    e = Engine(copy.deepcopy(ic), instr)
    _windows(o, e, 1.0, 2.0 if dim == 2 else 1.5)
    a, b = e.download(), o.download()
    s_a, s_b = (a.tau, b.tau) if deform == "finite" else (a.sig, b.sig)
    stress = np.linalg.norm(s_a - s_b) / np.linalg.norm(s_b)
    disp = np.linalg.norm(a.x - b.x) / np.linalg.norm(b.x - x0)
    ep = np.linalg.norm(a.epII[0] - b.epII[0]) / max(np.linalg.norm(b.epII[0]), 1e-300)
    print(f"{cons} {deform} {dim}d {precision}: stress {stress:.2e} displacement {disp:.2e} epII {ep:.2e}")
    assert stress < 1e-5 and disp < 1e-4 and ep < 1e-4
    if cons == "camC":
        ev = np.linalg.norm(a.epV - b.epV) / max(np.linalg.norm(b.epV), 1e-300)
        assert ev < 1e-4, ev
    e.close()


def test_mc_in_3d_is_rejected():
    from epgpu import Engine
    from epgpu.abi import EPError
    from epgpu.config import UnsupportedError
    from epgpu import ic_slump
    with pytest.raises((UnsupportedError, EPError)):
        ic, cfg = ic_slump(*C1_3D, plast={"status": True, "constitutive": "MC"})
        Engine(ic, cfg["instr"])
