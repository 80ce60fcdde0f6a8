"""Checkpoint snapshots: the fields of ``savlot`` as headless binary dumps.

The reference draws the fields named in ``instr["plot"]["what"]`` at every ``plot.freq`` checkpoint
when ``instr["plot"]["status"]`` is set (utils/savlot.jl:20-34 -> what_plot_field,
utils/plot.jl:27-135), as a scatter of the points at (x[1,:], x[end,:]).  Here the same fields are
evaluated on the device by ``epgpu_fields`` — only they cross the host link, not the whole state —
and written with the plot coordinates to one ``.npz`` file per checkpoint; no figure is drawn.

File layout (``snapshot_<t>.npz``, numpy's zip of ``.npy`` arrays): ``t`` (scalar), ``what`` (the
field names in request order), ``x`` and ``z`` (the plot coordinates, np values each), and one array of
np values per field, under the reference's option names ("P", "sigxx", "epsxx", "epII", "epV", "du",
"z0", "coh0", "phi0", "n0", "n", "J", "ms").
"""
from __future__ import annotations

import os

import numpy as np

# the bit order of EP_FIELD_* in include/epgpu.h
FIELDS = ("P", "sigxx", "epsxx", "epII", "epV", "du", "coh0", "phi0", "n", "J", "ms", "x", "z")
BITS = {name: 1 << i for i, name in enumerate(FIELDS)}
# plot.jl:112-117: the "n0" option shows mpts.n, the current porosity
ALIASES = {"n0": "n"}
# the reference's options (plot.jl:28-135); "z0" is the set-up z of each point, held on the host
OPTIONS = ("P", "sigxx", "epsxx", "epII", "epV", "du", "z0", "coh0", "phi0", "n0", "n", "J", "ms")


def mask(what) -> int:
    """EP_FIELD_* mask of a list of option names; an unknown name raises like plot.jl:137-138."""
    m = 0
    for w in what:
        if w == "z0":
            continue
        key = ALIASES.get(w, w)
        if key not in BITS:
            raise ValueError(f"UndefinedPlotOption: {w}")
        m |= BITS[key]
    return m


def rows(m: int) -> list:
    """Device field names of the rows that epgpu_fields writes for mask m, in order."""
    return [name for name in FIELDS if m & BITS[name]]


def collect(engine, what, z0=None) -> dict:
    """The requested options plus the plot coordinates, evaluated on the device."""
    names = list(what)
    got = engine.fields(rows(mask(names) | BITS["x"] | BITS["z"]))
    out = {"x": got["x"], "z": got["z"]}
    for w in names:
        if w == "z0":
            if z0 is None:
                raise ValueError("z0 is a set-up field: pass the host's mpts.z0")
            out[w] = np.asarray(z0, dtype=np.float64).copy()
        else:
            out[w] = got[ALIASES.get(w, w)]
    return out


def save(path: str, t: float, what, data: dict) -> str:
    np.savez(path, t=np.float64(t), what=np.array(list(what)), **data)
    return path


def load(path: str) -> dict:
    with np.load(path, allow_pickle=False) as f:
        out = {k: f[k] for k in f.files}
    out["t"] = float(out["t"])
    out["what"] = [str(w) for w in out["what"]]
    return out


def writer(out_dir: str, instr: dict, z0=None):
    """An ``on_checkpoint(t, engine)`` callback for the time-loop drivers of ``workflow``: writes
    ``out_dir/snapshot_<t>.npz`` with ``instr["plot"]["what"]`` when ``instr["plot"]["status"]``
    is set (the switch savlot reads), and nothing otherwise."""
    plot = instr.get("plot", {})
    what = list(plot.get("what", ()))
    mask(what)   # unknown options fail before the run, not at its first checkpoint
    os.makedirs(out_dir, exist_ok=True)
    written = []

    def on_checkpoint(t, engine):
        if not plot.get("status", False):
            return
        path = os.path.join(out_dir, f"snapshot_{t:012.6f}.npz")
        written.append(save(path, t, what, collect(engine, what, z0)))

    on_checkpoint.written = written
    return on_checkpoint
