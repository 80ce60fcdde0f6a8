"""Checkpoint snapshots (epgpu/snapshot.py): the savlot option names and their device field mask, the
writer callback and the file format, on the CPU with a stand-in for the device fields; and the
oracle restatement of plot.jl's field formulas on hand-made values."""
import numpy as np
import pytest


def test_mask_follows_the_header_bit_order():
    from epgpu import snapshot
    assert snapshot.FIELDS[snapshot.FIELDS.index("P")] == "P"
    assert snapshot.mask(["P"]) == 1 and snapshot.mask(["z"]) == 1 << 12
    assert snapshot.mask(["epII", "P"]) == snapshot.mask(["P", "epII"])
    assert snapshot.rows(snapshot.mask(["ms", "P", "x"])) == ["P", "ms", "x"]
    # n0 shows the current porosity (plot.jl:112-117); z0 lives on the host
    assert snapshot.mask(["n0"]) == snapshot.mask(["n"])
    assert snapshot.mask(["z0"]) == 0
    assert set(snapshot.OPTIONS) - {"z0", "n0"} <= set(snapshot.FIELDS)


def test_unknown_option_raises_like_the_reference():
    from epgpu import snapshot
    with pytest.raises(ValueError, match="UndefinedPlotOption: vorticity"):
        snapshot.mask(["P", "vorticity"])
    with pytest.raises(ValueError, match="UndefinedPlotOption"):
        snapshot.writer("/nonexistent-is-not-created", {"plot": {"status": True, "what": ["bad"]}})


class _FakeEngine:
    """Stands in for Engine.fields: row i of the device output is i + the point index."""

    def __init__(self, np_):
        self.np = np_
        self.calls = []

    def fields(self, names):
        from epgpu import snapshot
        self.calls.append(list(names))
        order = snapshot.rows(snapshot.mask(names))
        return {n: float(snapshot.FIELDS.index(n)) + np.arange(self.np, dtype=np.float64) for n in order}


def test_writer_writes_one_file_per_checkpoint(tmp_path):
    from epgpu import snapshot
    instr = {"plot": {"status": True, "freq": 1.0, "what": ["epII", "z0", "n0", "P"]}}
    z0 = np.linspace(0.0, 1.0, 7)
    cb = snapshot.writer(str(tmp_path), instr, z0=z0)
    eng = _FakeEngine(7)
    for t in (1.0, 2.0, 2.5):
        cb(t, eng)
    assert len(cb.written) == 3
    s = snapshot.load(cb.written[-1])
    assert s["t"] == 2.5 and s["what"] == ["epII", "z0", "n0", "P"]
    np.testing.assert_array_equal(s["z0"], z0)
    np.testing.assert_array_equal(s["epII"], snapshot.FIELDS.index("epII") + np.arange(7.0))
    np.testing.assert_array_equal(s["n0"], snapshot.FIELDS.index("n") + np.arange(7.0))
    np.testing.assert_array_equal(s["x"], snapshot.FIELDS.index("x") + np.arange(7.0))
    np.testing.assert_array_equal(s["z"], snapshot.FIELDS.index("z") + np.arange(7.0))
    # one device call per checkpoint, the coordinates always included, z0 never asked of the device
    assert all(set(c) == {"epII", "n", "P", "x", "z"} for c in eng.calls)


def test_writer_is_silent_when_plotting_is_off(tmp_path):
    from epgpu import snapshot
    cb = snapshot.writer(str(tmp_path), {"plot": {"status": False, "what": ["P"]}})
    cb(1.0, _FakeEngine(3))
    assert cb.written == [] and list(tmp_path.iterdir()) == []


def test_plot_oracle_formulas():
    import plot_oracle as po
    from types import SimpleNamespace
    sig2 = np.array([[-3.0e3, 1.0e3], [-5.0e3, 2.0e3], [7.0, 8.0]])
    m = SimpleNamespace(sig=sig2, u=np.array([[3.0, 0.0], [4.0, 1.0]]), rho=np.array([2.0, 3.0]),
                        Omega=np.array([0.5, 2.0]), c0=np.array([2.0e4, 4.0e3]), x=np.array([[1.0, 2.0], [3.0, 4.0]]))
    np.testing.assert_array_equal(po.plot_field(m, "P"), [4.0, -1.5])
    np.testing.assert_array_equal(po.plot_field(m, "sigxx"), [-3.0, 1.0])
    np.testing.assert_array_equal(po.plot_field(m, "du"), [5.0, 1.0])
    np.testing.assert_array_equal(po.plot_field(m, "ms"), [1.0, 6.0])
    np.testing.assert_array_equal(po.plot_field(m, "coh0"), [20.0, 4.0])
    m.sig = np.vstack([sig2, np.zeros((3, 2))])
    np.testing.assert_array_equal(po.plot_field(m, "P"), -(sig2[0] + sig2[1] + sig2[2]) / 3 / 1e3)
    x, z = po.plot_coords(m)
    np.testing.assert_array_equal(x, [1.0, 2.0])
    np.testing.assert_array_equal(z, [3.0, 4.0])
    with pytest.raises(ValueError, match="UndefinedPlotOption"):
        po.plot_field(m, "vorticity")


def test_writer_in_the_time_loop_with_the_oracle(tmp_path, oracle_mod):
    """The writer as the on_checkpoint callback of the time-loop drivers: one file per checkpoint of
    the reference's range t:freq:te, the last one holding the final state's fields."""
    import plot_oracle as po
    from epgpu import ic_slump, slump, snapshot
    ic, cfg = ic_slump([64.1584, 16.0396], [40, 10], nonloc={"status": False, "ls": 0.5})
    cfg["instr"]["plot"] = {"status": True, "freq": 0.5, "what": ["P", "epII", "z0", "n0"], "dims": (500.0, 250.0)}
    ic["time"]["te"] = 1.0
    cb = snapshot.writer(str(tmp_path), cfg["instr"], z0=ic["mpts"].z0)
    out = slump(ic, cfg, workflow="elastodynamic", on_checkpoint=cb,
                engine_factory=lambda a, b: oracle_mod.Oracle(a, b))
    assert [round(snapshot.load(f)["t"], 9) for f in cb.written] == [0.0, 0.5, 1.0]
    last = snapshot.load(cb.written[-1])
    fin = out["ic"]["mpts"]
    for opt in ("P", "epII", "n0"):
        np.testing.assert_array_equal(last[opt], po.plot_field(fin, opt))
    np.testing.assert_array_equal(last["x"], fin.x[0])
    np.testing.assert_array_equal(last["z"], fin.x[-1])
    np.testing.assert_array_equal(last["z0"], ic["mpts"].z0)
