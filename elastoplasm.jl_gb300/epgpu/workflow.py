"""Time-loop drivers: ``elastoplasm``, ``slump``, ``slump!``, ``collapse``.

Mirrors workflow/worflow.jl:23-141 and script/example/{slump,collapse}.jl.
The inner ``while T > t`` loop of each checkpoint window runs on the device
(``Engine.run`` -> ``epgpu_run``); this module only walks the checkpoint list,
which the reference builds as ``sort(collect(t:freq:te))`` with Julia range
semantics (worflow.jl:24,69).  Figures/dumps (``savlot``) are replaced by an
optional ``on_checkpoint(t, engine)`` callback.
"""
from __future__ import annotations

import copy

from .julia import frange

ELASTODYNAMIC, ELASTOPLASTIC = 0, 1


def _default_engine(ic, instr):
    from .engine import Engine
    return Engine(ic, instr)


def _phase(engine, phase: int, checks, tg: float, time: dict, on_checkpoint) -> int:
    """Walk one phase's checkpoint list.  The GPU engine takes the whole list in one call
    (``epgpu_run_checkpoints``); other engines (the oracle) are driven window by window."""
    if hasattr(engine, "run_checkpoints"):
        t, n = engine.run_checkpoints(phase, checks, tg, float(time["t"][0]), on_checkpoint)
        time["t"][0] = t
        return n
    steps = 0
    for T in checks:
        t, n = engine.run(phase, T, tg, float(time["t"][0]))
        time["t"][0] = t
        steps += n
        if on_checkpoint and on_checkpoint(t, engine):
            break
    return steps


def elastodynamic(engine, time: dict, instr: dict, on_checkpoint=None) -> int:
    """``elastodynamic!`` (worflow.jl:23-47): gravity ramp, no return map."""
    checks = sorted(frange(time["t"][0], instr["plot"]["freq"], time["te"]))
    return _phase(engine, ELASTODYNAMIC, checks, time["tg"], time, on_checkpoint)


def elastoplastic(engine, time: dict, instr: dict, on_checkpoint=None) -> int:
    """``elastoplastic!`` (worflow.jl:68-93): full gravity, with return map."""
    checks = sorted(frange(time["t"][0], instr["plot"]["freq"], time["t"][1]))
    return _phase(engine, ELASTOPLASTIC, checks, time["tg"], time, on_checkpoint)


def elastoplasm(ic: dict, cfg: dict, mode: str = "elastodynamic", engine_factory=None, on_checkpoint=None) -> dict:
    """``elastoplasm(ic, cfg; mode)`` (worflow.jl:113-141); mutates ``ic`` in place."""
    instr = cfg["instr"]
    make = engine_factory or _default_engine
    engine = make(ic, instr)
    steps = 0
    if mode == "elastodynamic":
        steps += elastodynamic(engine, ic["time"], instr, on_checkpoint)
    elif mode == "elastoplastic":
        steps += elastoplastic(engine, ic["time"], instr, on_checkpoint)
    elif mode == "all-in-one":
        steps += elastodynamic(engine, ic["time"], instr, on_checkpoint)
        steps += elastoplastic(engine, ic["time"], instr, on_checkpoint)
    else:
        raise ValueError(f"Invalid workflow: {mode}. Choose 'elastodynamic', 'elastoplastic' or 'all-in-one'.")
    engine.download(ic["mpts"])
    engine.download_mesh(ic["mesh"])
    engine.close()
    return {"ic": ic, "cfg": cfg, "steps": steps}


def slump(ic: dict, cfg: dict, workflow: str = "elastodynamic", **kw) -> dict:
    """``slump(ic, cfg; workflow)`` (script/example/slump.jl:73-79): works on deep copies."""
    out = elastoplasm(copy.deepcopy(ic), copy.deepcopy(cfg), mode=workflow, **kw)
    out["success"] = True
    return out


def slump_(ic: dict, cfg: dict, workflow: str = "elastodynamic", **kw) -> dict:
    """``slump!(ic, cfg; workflow)`` (slump.jl:103-109): mutates ``ic``."""
    out = elastoplasm(ic, cfg, mode=workflow, **kw)
    out["success"] = True
    return out


def collapse(ic: dict, cfg: dict, **kw) -> dict:
    """``collapse(ic, cfg)`` (script/example/collapse.jl:80-86): elastodynamic only."""
    out = elastoplasm(copy.deepcopy(ic), copy.deepcopy(cfg), **kw)
    out["success"] = True
    return out
