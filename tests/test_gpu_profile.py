"""Per-kernel device times (epgpu_profile / epgpu_profile_read).

The profiled step is the one-step graph captured with a CUDA event after every kernel: it must leave
the same state as the plain graph (bit for bit in the FP64 step and the deterministic mixed step) and
time every kernel of every step.
"""
import copy

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

C1 = ([64.1584, 64.1584 / 4.0], [40, 10])
KERNELS = {"fp64": {"p2g64", "solve64", "g2p64", "elast64"},
           "mixed_df": {"zero", "p2g", "g2p", "fbar", "cons"}}


@pytest.mark.parametrize("precision", ["fp64", "mixed_df"])
def test_profiled_steps_equal_the_graph_and_time_each_kernel(precision):
    from epgpu import Engine, ic_slump
    ic, cfg = ic_slump(*C1, nonloc={"status": False, "ls": 0.5})
    instr = copy.deepcopy(cfg["instr"])
    if precision != "fp64":
        instr["gpu"] = {"precision": precision, "jaumann": False, "deterministic": True}
    g = [0.0, -9.81]
    a = Engine(copy.deepcopy(ic), instr)
    b = Engine(copy.deepcopy(ic), instr)
    b.profile(True)
    n = 4
    for phase in (0, 1):                      # a phase change takes a new capture
        for _ in range(n):
            va = a.step(phase, 0.02, g)
            vb = b.step(phase, 0.02, g)
            assert np.array_equal(va, vb)
    kt = b.kernel_times()
    b.profile(False)
    b.step(1, 0.02, g)                        # back on the plain graph
    a.step(1, 0.02, g)
    sa, sb = a.download(), b.download()
    for f in ("x", "v", "tau", "Fij", "bij", "epII"):
        assert np.array_equal(np.asarray(getattr(sa, f)), np.asarray(getattr(sb, f))), f
    assert KERNELS[precision] <= set(kt), sorted(kt)
    for name, (launches, ms) in kt.items():
        assert launches % (2 * n) == 0 and launches > 0, (name, launches)
        assert 0.0 < ms < 1e3, (name, ms)
    a.close()
    b.close()
