"""Host logic of bench.py that needs no GPU: the clock record (median SM clock under load, maximum
clock, throttle reasons) read back from nvidia-smi's CSV lines, and the CFL time step."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    sys.path.insert(0, ROOT)
    import bench
    return bench


def test_clock_record_from_sampler_lines(tmp_path, monkeypatch):
    bench = _bench()
    monkeypatch.setattr(bench.Clocks, "out_dir", str(tmp_path))
    c = bench.Clocks(0)
    # index, clocks.sm, clocks.max.sm, power.draw, reasons.active, hw_slowdown, hw_thermal, sw_thermal, sw_power_cap
    lines = ["0, 2070, 2070, 700.1, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
             "0, 1980, 2070, 1390.5, 0x0000000000000004, Not Active, Not Active, Not Active, Active",
             "0, 2070, 2070, 900.0, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
             "[N/A] garbled line",
             ""]
    with open(c.path, "w") as f:
        f.write("\n".join(lines))
    s = c.summary()
    assert s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == ["sw_power_cap"]


def test_clock_record_without_samples(tmp_path, monkeypatch):
    bench = _bench()
    monkeypatch.setattr(bench.Clocks, "out_dir", str(tmp_path))
    c = bench.Clocks(0)
    open(c.path, "w").close()
    assert c.summary() == {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}


def test_cfl_dt_follows_the_reference_rule():
    """get_dt (physics.jl:21-26) without the checkpoint clip: 0.5 max_d h_d / (vmax_d + c) -- the
    reference takes the maximum over the directions, not the minimum."""
    bench = _bench()

    class Mesh:
        dim = 2
        h = [0.1, 0.2]

    dt = bench.cfl_dt(Mesh(), {"c": 100.0}, [1.0, 0.0])
    assert abs(dt - 0.5 * max(0.1 / 101.0, 0.2 / 100.0)) < 1e-15
