"""Parity at the scaled-up 2d slump as the reference builds it: nel=[640,160], 3x3 points per cell
(365,024 points, 103,201 nodes), cubic B-spline, finite strain, FLIP with mUSL, F-bar, damping 0.1,
Drucker-Prager with softening, the seeded exponential-covariance cohesion field (mean 20 kPa, CoV 0.3,
5 m, >= 1 kPa), nonlocal averaging off.

The state is settled for 0.5 s of elastoplastic flow by the FP64 device step (the drop-in, whose
bitwise agreement with the oracle the first test checks at this size), so that tens of thousands of
points yield.  From that state the oracle runs single-threaded (its scatters are then in ascending
point order, so its result does not depend on thread timing) for STEPS elastoplastic steps with the
reference's CFL rule; every device run replays the oracle's dt sequence.

Bounds (written here, the benchmark spec targets): FP64 step 1e-10 relative per field; mixed and
mixed_df with the exact return map: stress 1e-5, displacement 1e-4 and runout 1e-4 relative, the
error measures of test_gpu_mixed.errors (runout = displacement of the largest x since t = 0).
"""
import copy

import numpy as np
import pytest

from conftest import compare_points
from test_gpu_mixed import errors

pytestmark = pytest.mark.gpu

L2 = [64.1584, 16.0396]
NEL2 = [640, 160]
SETTLE = 0.5
STEPS = 35
FP64_STEPS = 5
RTOL_FP64 = 1e-10
STRESS_TOL, DISP_TOL, RUNOUT_TOL = 1e-5, 1e-4, 1e-4


def _workload():
    from epgpu import ic_slump
    fw = {"deform": "finite", "trsfr": "std", "C_pf": 1.0, "musl": True, "locking": True, "damping": 0.1}
    grf = {"status": True, "covariance": "exponential",
           "param": {"Ix": [5.0, 5.0], "mean": 2.0e4, "cov": 0.3, "min": 1.0e3, "seed": 1234}}
    return ic_slump(L2, NEL2, ni=3, fwrk=fw, nonloc={"status": False, "ls": 0.5}, grf=grf)


def _cfl(mesh, cmpr, vmax):
    # get_dt (physics.jl:21-26) without the checkpoint clip
    return 0.5 * max(mesh.h[i] / (vmax[i] + cmpr["c"]) for i in range(mesh.dim))


@pytest.fixture(scope="module")
def c2_runs(oracle_mod):
    from epgpu import Engine
    ic, cfg = _workload()
    x0 = ic["mpts"].x.copy()
    e = Engine(copy.deepcopy(ic), cfg["instr"])
    t, n = e.run(1, SETTLE, 10.0, 0.0)
    s0 = e.download()
    e.close()
    assert t == SETTLE and n > 100
    o = oracle_mod.Oracle({**ic, "mpts": s0.copy()}, cfg["instr"], threads=1)
    g = [0.0, -9.81]
    vm, dts, snaps = s0.vmax.copy(), [], {}
    for k in range(STEPS):
        dts.append(_cfl(ic["mesh"], ic["cmpr"], vm))
        vm = o.step(1, dts[-1], g)
        if k + 1 in (FP64_STEPS, STEPS):
            snaps[k + 1] = o.download()
    o.close()
    return {"ic": ic, "cfg": cfg, "x0": x0, "s0": s0, "dts": dts, "snaps": snaps}


def _replay(runs, instr, nsteps):
    from epgpu import Engine
    ic = {**runs["ic"], "mpts": runs["s0"].copy()}
    e = Engine(ic, instr)
    for dt in runs["dts"][:nsteps]:
        e.step(1, dt, [0.0, -9.81])
    out = e.download()
    e.close()
    return out


def test_fp64_step_matches_single_thread_oracle_c2(c2_runs):
    b = c2_runs["snaps"][FP64_STEPS]
    assert (b.dlam != 0).sum() > 1000             # the plastic branch runs at this size
    a = _replay(c2_runs, c2_runs["cfg"]["instr"], FP64_STEPS)
    worst = compare_points(a, b, RTOL_FP64)
    assert np.array_equal(a.p2e, b.p2e)
    print(f"c2 FP64 step, {FP64_STEPS} plastic steps: max rel diff {max(worst.values()):.2e}, "
          f"{int((b.dlam != 0).sum())} plastic points")


@pytest.mark.parametrize("precision", ["mixed", "mixed_df"])
def test_mixed_exact_map_vs_oracle_c2(c2_runs, precision):
    instr = copy.deepcopy(c2_runs["cfg"]["instr"])
    instr["gpu"] = {"precision": precision, "jaumann": False}
    a = _replay(c2_runs, instr, STEPS)
    b = c2_runs["snaps"][STEPS]
    s, d, r = errors(a, b, c2_runs["x0"])
    print(f"c2 {precision} exact map, {STEPS} plastic steps: stress {s:.3e} displacement {d:.3e} runout {r:.3e} "
          f"({int((b.dlam != 0).sum())} plastic points)")
    assert s <= STRESS_TOL and d <= DISP_TOL and r <= RUNOUT_TOL
