"""Parity of the CUDA step (through the C ABI) with the FP64 CPU oracle.

The FP64 device step adds every nodal sum in ascending point order and
compiles without multiply-add contraction, so it is expected to match the
oracle bit for bit; the tolerance written in these tests is the one the
drop-in is held to, 1e-10 relative (per field, scaled by the field's
magnitude), and the measured difference is reported.
"""
import copy
import ctypes as C

import numpy as np
import pytest

from conftest import POINT_FIELDS, compare_points

pytestmark = pytest.mark.gpu

RTOL_FP64 = 1e-10
C1 = ([64.1584, 64.1584 / 4.0], [40, 10])
C1_3D = ([64.1584, 64.1584 / 4.0, 64.1584 / 4.0], [40, 10, 10])


def _engine(ic, instr):
    from epgpu import Engine
    return Engine(ic, instr)


def _pair(ic, instr, oracle_mod):
    return oracle_mod.Oracle(copy.deepcopy(ic), instr), _engine(copy.deepcopy(ic), instr)


def _run_both(o, e, phase, T, t, tg=10.0):
    to, no = o.run(phase, T, tg, t)
    te, ne = e.run(phase, T, tg, t)
    assert (to, no) == (te, ne), ((to, no), (te, ne))
    return te


def test_step_by_step_config1(oracle_mod):
    from epgpu import ic_slump
    ic, cfg = ic_slump(*C1)
    o, e = _pair(ic, cfg["instr"], oracle_mod)
    g = [0.0, -9.81]
    for k in range(5):
        vo = o.step(1 if k >= 3 else 0, 0.03, g)
        ve = e.step(1 if k >= 3 else 0, 0.03, g)
        assert np.array_equal(vo, ve)
        compare_points(e.download(), o.download(), RTOL_FP64)
    mo, me = o.download_mesh(), e.download_mesh()
    for f in ("mi", "p", "v", "a", "oobf"):
        assert np.array_equal(getattr(mo, f), getattr(me, f)), f
    assert np.array_equal(mo.dJ[0], me.dJ[0])


def test_run_windows_config1(oracle_mod):
    # elastodynamic then elastoplastic windows with nonlocal averaging and DP softening
    from epgpu import ic_slump
    ic, cfg = ic_slump(*C1)
    o, e = _pair(ic, cfg["instr"], oracle_mod)
    t = _run_both(o, e, 0, 1.0, 0.0)
    worst = compare_points(e.download(), o.download(), RTOL_FP64)
    t = _run_both(o, e, 1, 2.0, t)
    a, b = e.download(), o.download()
    assert (b.dlam != 0).sum() > 50          # the plastic branch and nonlocal pass are exercised
    worst = compare_points(a, b, RTOL_FP64)
    assert np.array_equal(a.p2e, b.p2e) and np.array_equal(a.p2n, b.p2n)
    print("max rel diff", max(worst.values()))


# the 12 cases of test/testset/test_slump.jl:3-16
SWITCHES = [(d, t, lk) for d in ("finite", "infinitesimal") for t in ("std", "tpic", "apic") for lk in (True, False)]
APIC_FIELDS = POINT_FIELDS + ["Bij", "Dij"]


@pytest.mark.parametrize("deform,trsfr,locking", SWITCHES)
def test_switch_matrix(oracle_mod, deform, trsfr, locking):
    from epgpu import ic_slump
    fw = {"deform": deform, "trsfr": trsfr, "C_pf": 0.99, "musl": True, "locking": locking, "damping": 0.1}
    ic, cfg = ic_slump(*C1, fwrk=fw, nonloc={"status": True, "ls": 0.5})
    o, e = _pair(ic, cfg["instr"], oracle_mod)
    t = _run_both(o, e, 0, 1.0, 0.0)
    t = _run_both(o, e, 1, 1.5, t)
    a, b = e.download(), o.download()
    compare_points(a, b, RTOL_FP64, fields=APIC_FIELDS if trsfr == "apic" else POINT_FIELDS)
    if trsfr == "apic":
        assert np.abs(np.asarray(b.Bij)).max() > 1e-3 and np.abs(np.asarray(b.Dij)).max() > 0


@pytest.mark.parametrize("basis", [{"which": "gimpm", "how": "undeformed", "ghost": True},
                                   {"which": "smpm", "how": None, "ghost": False},
                                   {"which": "gimpm", "how": "detFij", "ghost": True}])
def test_other_bases(oracle_mod, basis):
    from epgpu import ic_slump
    ic, cfg = ic_slump(*C1, basis=basis)
    o, e = _pair(ic, cfg["instr"], oracle_mod)
    t = _run_both(o, e, 0, 1.0, 0.0)
    t = _run_both(o, e, 1, 1.5, t)
    compare_points(e.download(), o.download(), RTOL_FP64)


def test_full_all_in_one_config1(oracle_mod):
    # configs[0]: the reference's CPU-runnable case, whole workflow (15 s simulated)
    from epgpu import ic_slump, slump
    ic, cfg = ic_slump(*C1)
    out_g = slump(ic, cfg, workflow="all-in-one")
    out_o = slump(ic, cfg, workflow="all-in-one", engine_factory=lambda a, b: oracle_mod.Oracle(a, b))
    assert out_g["steps"] == out_o["steps"] and out_g["steps"] > 400
    assert out_g["ic"]["time"]["t"][0] == out_o["ic"]["time"]["t"][0]
    worst = compare_points(out_g["ic"]["mpts"], out_o["ic"]["mpts"], RTOL_FP64)
    print("all-in-one steps", out_g["steps"], "max rel diff", max(worst.values()))


@pytest.mark.parametrize("kw", [
    {},
    {"basis": {"which": "gimpm", "how": "undeformed", "ghost": True},
     "fwrk": {"deform": "infinitesimal", "trsfr": "tpic", "C_pf": 0.0, "musl": False, "locking": False,
              "damping": 0.1},
     "plast": {"status": True, "constitutive": "J2"}, "nonloc": {"status": False, "ls": 0.5}},
    {"fwrk": {"deform": "finite", "trsfr": "apic", "C_pf": 0.99, "musl": True, "locking": True, "damping": 0.1},
     "nonloc": {"status": False, "ls": 0.5}},
])
def test_3d(oracle_mod, kw):
    from epgpu import ic_slump
    over = {"c0": 5.0e4, "Hp": 1.0e5} if "plast" in kw else None
    ic, cfg = ic_slump(*C1_3D, cmpr_over=over, **kw)
    if over:
        ic["mpts"].c0[:] = 5.0e4
    o, e = _pair(ic, cfg["instr"], oracle_mod)
    t = _run_both(o, e, 0, 0.3, 0.0)
    t = _run_both(o, e, 1, 0.5, t)
    apic = kw.get("fwrk", {}).get("trsfr") == "apic"
    compare_points(e.download(), o.download(), RTOL_FP64, fields=APIC_FIELDS if apic else POINT_FIELDS)


def test_collapse_convergence_gpu():
    from epgpu import collapse, ic_collapse
    fw = {"deform": "finite", "trsfr": "std", "C_pf": 1.0, "musl": True, "locking": False, "damping": 0.1}
    errs = [np.inf]
    for nz in (5, 10, 20, 40):
        ic, cfg = ic_collapse([5, nz], 0.0, 1.0e4, 80.0, 50.0, fwrk=fw, nonloc={"status": False, "ls": 0.5})
        z0 = ic["mpts"].x[-1].copy()
        out = collapse(ic, cfg)
        m, cm = out["ic"]["mpts"], out["ic"]["cmpr"]
        x = np.abs(cm["rho0"] * 9.81 * (50.0 - z0))
        err = np.sum(np.abs(np.abs(m.sig[1]) - x) * m.Omega0) / (9.81 * cm["rho0"] * 50.0 * np.sum(m.Omega0))
        assert err < errs[-1]
        errs.append(err)
    assert errs[-1] < 2e-3


def test_edge_point_outside_domain(oracle_mod):
    # a point left of x = 0 is clamped into the first element (tplgy.jl:134-136)
    from epgpu import ic_slump
    ic, cfg = ic_slump(*C1)
    ic["mpts"].x[0, 0] = -0.05
    o, e = _pair(ic, cfg["instr"], oracle_mod)
    g = [0.0, -9.81]
    o.step(0, 0.02, g)
    e.step(0, 0.02, g)
    a, b = e.download(), o.download()
    assert a.p2e[0] == 1
    compare_points(a, b, RTOL_FP64)


def test_nonfinite_point_is_reported():
    from epgpu import ic_slump
    from epgpu.abi import EPError
    ic, cfg = ic_slump(*C1)
    ic["mpts"].x[1, 7] = np.nan
    e = _engine(ic, cfg["instr"])
    with pytest.raises(EPError) as ex:
        e.step(0, 0.02, [0.0, -9.81])
    assert ex.value.status == 3
    # the handle stays usable: the state can still be read back
    assert e.download().nmp == ic["mpts"].nmp


def test_invalid_bspline_position_matches_reference_error(oracle_mod):
    # bsmpm on a ghost-padded mesh: nodes outside xB have no B-spline class (bsmpm.jl:75)
    from epgpu import ic_slump
    from epgpu.abi import EPError
    ic, cfg = ic_slump(*C1, basis={"which": "bsmpm", "how": None, "ghost": True})
    o = oracle_mod.Oracle(copy.deepcopy(ic), cfg["instr"])
    with pytest.raises(EPError) as eo:
        o.step(0, 0.02, [0.0, -9.81])
    e = _engine(copy.deepcopy(ic), cfg["instr"])
    with pytest.raises(EPError) as eg:
        e.step(0, 0.02, [0.0, -9.81])
    assert eo.value.status == eg.value.status == 7


def test_empty_point_set():
    from epgpu import ic_slump
    from epgpu.ic import Point
    ic, cfg = ic_slump(*C1)
    m = ic["mpts"]
    sel = np.zeros(m.nmp, dtype=bool)
    kw = {}
    for k, v in m.__dict__.items():
        if isinstance(v, np.ndarray) and v.shape and v.shape[-1] == m.nmp:
            kw[k] = np.asfortranarray(v[..., sel])
        else:
            kw[k] = v
    kw["nmp"] = 0
    ic["mpts"] = Point(**kw)
    e = _engine(ic, cfg["instr"])
    v = e.step(1, 0.02, [0.0, -9.81])
    assert np.array_equal(v, [0.0, 0.0])
    assert e.download_mesh().mi.sum() == 0.0


def test_bin_cells_standalone_config2():
    # the stand-alone counting sort at the full nel=[640,160], 365,024-point size
    import torch
    from epgpu import abi, ic_slump
    ic, _ = ic_slump([64.1584, 16.0396], [640, 160], ni=3)
    m, p = ic["mesh"], ic["mpts"]
    rng = np.random.default_rng(5)
    x = p.x + rng.normal(scale=0.3, size=p.x.shape)           # off-lattice points, some outside
    xd = torch.tensor(np.ascontiguousarray(x), dtype=torch.float64, device="cuda")   # direction-major
    n = p.nmp
    nc = m.nel[0] * m.nel[1]
    p2e = torch.empty(n, dtype=torch.int32, device="cuda")
    start = torch.empty(nc + 1, dtype=torch.int32, device="cuda")
    lst = torch.empty(n, dtype=torch.int32, device="cuda")
    lib = abi.load_library()
    nel = (C.c_int64 * 3)(*m.nel[:2], 0)
    h = (C.c_double * 3)(*m.h, 0.0)
    x0 = (C.c_double * 3)(*m.x0, 0.0)
    for _ in range(2):
        st = lib.epgpu_bin_cells(2, nel, h, x0, C.c_void_p(xd.data_ptr()), n, C.c_void_p(p2e.data_ptr()),
                                 C.c_void_p(start.data_ptr()), C.c_void_p(lst.data_ptr()), None)
        assert st == 0
    # expected cell: clamp(fld(x - x0, h), 0, nel-1) with Python's exact float floor division
    e = [np.clip(np.floor_divide(x[d] - m.x0[d], m.h[d]), 0, m.nel[d] - 1).astype(np.int64) for d in range(2)]
    want = e[1] + m.nel[1] * e[0]
    got = p2e.cpu().numpy()
    assert np.array_equal(got, want)
    counts = np.bincount(want, minlength=nc)
    assert np.array_equal(start.cpu().numpy(), np.concatenate([[0], np.cumsum(counts)]))
    order = np.argsort(want, kind="stable")
    assert np.array_equal(lst.cpu().numpy(), order)
