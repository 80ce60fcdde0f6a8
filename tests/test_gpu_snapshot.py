"""epgpu_fields (savlot's plot fields evaluated on the device) against the restatement of plot.jl
(oracle/plot_oracle.py) applied to the full downloaded state: identical bits, 2d and 3d, FP64 and
mixed; and the checkpoint writer driven by the time loop."""
import copy

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

C1 = ([64.1584, 64.1584 / 4.0], [40, 10])
C1_3D = ([64.1584, 16.0396, 16.0396], [16, 4, 4])


@pytest.mark.parametrize("dim,precision", [(2, "fp64"), (2, "mixed_df"), (3, "fp64"), (3, "mixed")])
def test_device_fields_match_plot_formulas(dim, precision):
    import plot_oracle as po
    from epgpu import Engine, ic_slump, snapshot
    L, nel = C1 if dim == 2 else C1_3D
    ic, cfg = ic_slump(L, nel, nonloc={"status": False, "ls": 0.5})
    rng = np.random.default_rng(3)
    ic["mpts"].u[...] = rng.normal(size=ic["mpts"].u.shape)        # passed through by the step
    ic["mpts"].epV[...] = rng.normal(size=ic["mpts"].epV.shape)
    instr = copy.deepcopy(cfg["instr"])
    instr["gpu"] = {"precision": precision, "jaumann": False}
    e = Engine(copy.deepcopy(ic), instr)
    t = 0.0
    for phase, T in ((0, 0.5), (1, 0.8)):
        t, _ = e.run(phase, T, 10.0, t)
    got = e.fields(snapshot.FIELDS)
    full = e.download()
    e.close()
    for opt in snapshot.OPTIONS:
        if opt == "z0":
            continue
        want = po.plot_field(full, opt) if opt != "phi0" else np.asarray(ic["mpts"].phi)
        have = got[snapshot.ALIASES.get(opt, opt)]
        assert np.array_equal(have, want), (opt, float(np.abs(have - want).max()))
    x, z = po.plot_coords(full)
    assert np.array_equal(got["x"], x) and np.array_equal(got["z"], z)
    assert np.abs(got["P"]).max() > 0 and np.abs(got["du"]).max() > 0


def test_snapshot_writer_in_the_time_loop(tmp_path):
    import plot_oracle as po
    from epgpu import ic_slump, slump, snapshot
    ic, cfg = ic_slump(*C1, nonloc={"status": False, "ls": 0.5})
    cfg["instr"]["gpu"] = {"precision": "mixed_df", "jaumann": False}
    cfg["instr"]["plot"] = {"status": True, "freq": 0.5, "what": ["P", "epII", "z0", "J"], "dims": (500.0, 250.0)}
    ic["time"]["te"] = 1.0
    cb = snapshot.writer(str(tmp_path), cfg["instr"], z0=ic["mpts"].z0)
    out = slump(ic, cfg, workflow="elastodynamic", on_checkpoint=cb)
    assert len(cb.written) == 3             # checkpoints 0.0, 0.5, 1.0 (worflow.jl:24)
    last = snapshot.load(cb.written[-1])
    fin = out["ic"]["mpts"]
    assert last["t"] == pytest.approx(1.0)
    for opt in ("P", "epII", "J"):
        assert np.array_equal(last[opt], po.plot_field(fin, opt)), opt
    np.testing.assert_array_equal(last["z0"], ic["mpts"].z0)
