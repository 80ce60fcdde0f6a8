"""The checkpoint-list entry point (``epgpu_run_checkpoints``): one call per workflow phase, the
reference's ``for T in sort(collect(t:freq:te)); while T > t ... end; savlot(...) end``
(worflow.jl:23-47, 68-93) with the callback in place of savlot.

It is held to the per-window calls of ``epgpu_run`` (and through them to the FP64 oracle): the same
steps, the same times and the same bits at every checkpoint.
"""
import copy

import numpy as np
import pytest

from conftest import compare_points

pytestmark = pytest.mark.gpu

C1 = ([64.1584, 64.1584 / 4.0], [40, 10])


def _ic(**kw):
    from epgpu import ic_slump
    return ic_slump(*C1, **kw)


def test_checkpoint_list_matches_the_oracle_windows(oracle_mod):
    from epgpu import Engine
    from epgpu.julia import frange
    ic, cfg = _ic()
    instr = cfg["instr"]
    checks = sorted(frange(0.0, 0.25, 1.0))            # 0.0, 0.25, ..., 1.0 as worflow.jl:24 builds it
    o = oracle_mod.Oracle(copy.deepcopy(ic), instr)
    e = Engine(copy.deepcopy(ic), instr)
    seen = []

    def cb(t, eng):
        seen.append((t, eng.download()))

    t_gpu, n_gpu = e.run_checkpoints(0, checks[::-1], 10.0, 0.0, cb)   # the library sorts the list
    t, n_or = 0.0, 0
    for k, T in enumerate(checks):
        t, n = o.run(0, T, 10.0, t)
        n_or += n
        assert seen[k][0] == t, (k, seen[k][0], t)
        compare_points(seen[k][1], o.download(), 1e-10)
    assert (t_gpu, n_gpu) == (t, n_or)
    assert len(seen) == len(checks)                     # the window T = t = 0 takes no step but is reported
    e.close()


def test_checkpoint_list_equals_per_window_runs_mixed():
    """The mixed step in deterministic mode: one call over the list ends in the bits of the per-window
    calls, for both phases."""
    from epgpu import Engine
    ic, cfg = _ic(nonloc={"status": False, "ls": 0.5})
    instr = copy.deepcopy(cfg["instr"])
    instr["gpu"] = {"precision": "mixed_df", "jaumann": False, "deterministic": True}
    a = Engine(copy.deepcopy(ic), instr)
    b = Engine(copy.deepcopy(ic), instr)
    plan = ((0, [0.5, 1.0, 1.5]), (1, [1.75, 2.0]))
    t_a = t_b = 0.0
    for phase, checks in plan:
        t_a, _ = a.run_checkpoints(phase, checks, 10.0, t_a)
        for T in checks:
            t_b, _ = b.run(phase, T, 10.0, t_b)
        assert t_a == t_b
    compare_points(a.download(), b.download(), 0.0)
    a.close()
    b.close()


def test_callback_stops_the_phase_and_errors_propagate():
    from epgpu import Engine
    from epgpu.abi import EPError
    ic, _cfg = _ic()
    e = Engine(copy.deepcopy(ic), _cfg["instr"])
    calls = []
    t, n = e.run_checkpoints(0, [0.2, 0.4, 0.6], 10.0, 0.0, lambda t, eng: calls.append(t) or len(calls) == 2)
    assert len(calls) == 2 and t == calls[-1] and t >= 0.4 and n > 0

    def boom(t, eng):
        raise KeyError("raised in the callback")

    with pytest.raises(KeyError):
        e.run_checkpoints(0, [0.8], 10.0, t, boom)
    with pytest.raises(EPError):
        e.run_checkpoints(0, [np.nan], 10.0, t)
    e.close()
