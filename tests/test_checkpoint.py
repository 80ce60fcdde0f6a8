"""Checkpoint / resume (epgpu/checkpoint.py) on the CPU with the FP64 oracle: the file gives back every
array bit for bit, and a run interrupted at a checkpoint and resumed from the file ends in exactly the
state of the uninterrupted run."""
import copy

import numpy as np
import pytest

from conftest import POINT_FIELDS, compare_points


def test_file_round_trip(tmp_path):
    from epgpu import checkpoint, ic_slump
    ic, cfg = ic_slump([64.1584, 16.0396], [40, 10])
    ic["mpts"].v[...] = np.random.default_rng(0).normal(size=ic["mpts"].v.shape)
    path = checkpoint.save(str(tmp_path / "s.npz"), ic["mpts"], ic["time"])
    m, time = checkpoint.load(path)
    for k, v in ic["mpts"].__dict__.items():
        w = getattr(m, k)
        if isinstance(v, np.ndarray):
            assert w.dtype == v.dtype and w.shape == v.shape and np.array_equal(w, v), k
            assert w.flags.f_contiguous == v.flags.f_contiguous or v.ndim == 1, k
        else:
            assert w == v, k
    assert set(time) == set(ic["time"])
    assert np.array_equal(time["t"], ic["time"]["t"]) and time["te"] == ic["time"]["te"]


@pytest.mark.parametrize("trsfr", ["std", "tpic", "apic"])
def test_resume_continues_bit_for_bit(tmp_path, oracle_mod, trsfr):
    """TPIC carries the previous step's ∇v and APIC its Bᵢⱼ from one step to the next: the file must
    hold them for the resumed run to match."""
    from epgpu import checkpoint, ic_slump
    fw = {"deform": "finite", "trsfr": trsfr, "C_pf": 0.99, "musl": True, "locking": True, "damping": 0.1}
    ic, cfg = ic_slump([64.1584, 16.0396], [40, 10], fwrk=fw, nonloc={"status": True, "ls": 0.5})
    # uninterrupted: 1.0 s elastic, then plastic to 1.6 s
    o = oracle_mod.Oracle(copy.deepcopy(ic), cfg["instr"])
    t, _ = o.run(0, 1.0, 10.0, 0.0)
    mid = o.download()
    t, _ = o.run(1, 1.6, 10.0, t)
    ref = o.download()
    # interrupted at t = 1.0, written, read back into a new context, continued
    time = dict(ic["time"])
    time["t"] = np.array([1.0, ic["time"]["t"][1]])
    path = checkpoint.save(str(tmp_path / "mid.npz"), mid, time)
    m, time2 = checkpoint.load(path)
    ic2 = dict(ic)
    ic2["mpts"] = m
    o2 = oracle_mod.Oracle(ic2, cfg["instr"])
    t2, _ = o2.run(1, 1.6, 10.0, float(time2["t"][0]))
    assert t2 == t
    extra = ["Bij", "Dij"] if trsfr == "apic" else []
    compare_points(o2.download(), ref, 0.0, fields=POINT_FIELDS + ["epV", "c0", "phi", "Omega0", "rho0"] + extra)
