"""Checkpoint / resume: the whole point state and the time record in one file.

The reference keeps its state only in the NamedTuple that ``elastoplasm`` returns (worflow.jl:140) and
has no restart file.  Here a checkpoint is the downloaded ``Point`` (every array of ``ep_mpts_view``,
``z0`` and the topology) with the ``time`` record, written as a numpy ``.npz`` (headless, one array per
field, no pickled objects); loading it gives the arrays back bit for bit, so uploading them continues the
run from the same state (``epgpu_upload`` is the resume).

    from epgpu import checkpoint
    checkpoint.save("state.npz", engine.download(), ic["time"])      # at any checkpoint
    mpts, time = checkpoint.load("state.npz")
    ic["mpts"], ic["time"] = mpts, time                                # then Engine(ic, instr) or upload
"""
from __future__ import annotations

import dataclasses

import numpy as np

from .ic import Point

_SCALARS = ("ndim", "nmp")


def save(path: str, mpts: Point, time: dict | None = None) -> str:
    arrays = {}
    for f in dataclasses.fields(Point):
        v = getattr(mpts, f.name)
        if f.name in _SCALARS:
            arrays[f.name] = np.int64(v)
        elif v is not None:
            arrays["p_" + f.name] = np.asarray(v)
    for k, v in (time or {}).items():
        arrays["t_" + k] = np.asarray(v)
    np.savez(path, **arrays)
    return path


def load(path: str):
    """(Point, time dict) from a checkpoint file; arrays keep their dtype, shape and column-major order."""
    with np.load(path, allow_pickle=False) as f:
        data = {k: f[k] for k in f.files}
    kw = {}
    for fl in dataclasses.fields(Point):
        if fl.name in _SCALARS:
            kw[fl.name] = int(data[fl.name])
        elif "p_" + fl.name in data:
            kw[fl.name] = np.asfortranarray(data["p_" + fl.name])
        else:
            kw[fl.name] = None
    time = {}
    for k, v in data.items():
        if k.startswith("t_"):
            time[k[2:]] = v.copy() if v.ndim else v.item()
    return Point(**kw), time
