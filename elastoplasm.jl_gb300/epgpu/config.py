"""Configuration defaults and merge rules of ElastoPlasm (``require``/``kwargser``).

Mirrors api/require.jl:34-88 (defaults) and api/kwargser.jl:31-62 (merge).
The merge is *top level only*, exactly as the reference: passing
``fwrk={"deform": "infinitesimal"}`` replaces the whole ``fwrk`` group, so the
other ``fwrk`` keys disappear (kwargser.jl:34-36).  Unknown top-level keys are
reported with a warning and dropped (kwargser.jl:38-41).

The reference attaches a kernel table ``instr.cairn`` to the result
(kwargser.jl:49-60).  Here the same switches select the kernels of the CUDA
library instead; :func:`to_abi` turns the switches into the ``ep_cfg`` the
C-ABI expects and raises the errors the reference's ``init_*`` functions raise
for unsupported choices.
"""
from __future__ import annotations

import copy
import warnings

import numpy as np


def require(what: str = "instr") -> dict:
    """Default instruction set (api/require.jl:34-88)."""
    if what != "instr":
        raise ValueError(f"UnsupportedSymbol: {what}")
    return {
        "dtype": 64,
        "basis": {"which": "bsmpm", "how": None, "ghost": False},
        "fwrk": {"deform": "finite", "trsfr": "std", "C_pf": 1.0, "musl": True,
                 "locking": True, "damping": 0.1},
        "bcs": {"dirichlet": np.array([["roller", "roller"]] * 3, dtype=object)},
        "grf": {"status": False, "covariance": "gaussian",
                "param": {"Ix": [2.5, 2.5, 2.5], "Nh": 5000, "km": 100}},
        "plast": {"status": False, "constitutive": "DP"},
        "nonloc": {"status": True, "ls": 0.5},
        "plot": {"status": True, "freq": 1.0, "what": ["epII"], "dims": (500.0, 250.0)},
        "perf": {"status": False},
        # GB300 build switches (absent from the reference; defaults keep its behaviour)
        "gpu": {"precision": "fp64", "jaumann": False, "deterministic": False},
    }


def kwargser(kwargs: dict | None = None, dim: int = 2) -> dict:
    """Top-level merge of user switches over the defaults (api/kwargser.jl:31-62)."""
    kwargs = dict(kwargs or {})
    ref = require("instr")
    unused = [k for k in kwargs if k not in ref]
    if unused:
        warnings.warn("miscellaneous kwargs for require():" + "".join(f"\n\t- {k}" for k in unused))
    instr = copy.deepcopy(ref)
    for k, v in kwargs.items():
        if k in ref:
            instr[k] = copy.deepcopy(v)
    if instr["dtype"] not in (64, 32):
        raise ValueError(f"unsupported dtype {instr['dtype']}")
    instr["dim"] = int(dim)
    # validate the switches the way the reference's init_* functions do
    to_abi(instr)
    return instr


# --- enums shared with include/epgpu.h ------------------------------------------------
BASIS = {"bsmpm": 0, "gimpm": 1, "smpm": 2}
HOW = {None: 0, "undeformed": 1, "detFij": 2, "Fii": 3, "Uii": 4,
       "detΔFij": 5, "ΔFii": 6, "ΔUii": 7}
DEFORM = {"finite": 0, "infinitesimal": 1}
TRSFR = {"std": 0, "tpic": 1, "apic": 2}
CONSTITUTIVE = {"DP": 0, "J2": 1, "MC": 2, "camC": 3}
PRECISION = {"fp64": 0, "mixed": 1, "mixed_df": 2}


class UnsupportedError(ValueError):
    """A switch combination the reference rejects or this build leaves out."""


def to_abi(instr: dict) -> dict:
    """Translate switches into the integer fields of ``ep_cfg``."""
    b, f = instr["basis"], instr["fwrk"]
    dim = instr.get("dim", 2)
    if dim not in (2, 3):
        raise UnsupportedError(f"{dim}d workflow is not built (2d and 3d are)")
    if b.get("which") not in BASIS:
        raise UnsupportedError(f"{b.get('which')} is not a supported shape function basis")
    trsfr = f.get("trsfr")
    if trsfr not in TRSFR:
        raise UnsupportedError(f"{trsfr} is an unsupported transfer scheme")
    if f.get("deform") not in DEFORM:
        raise UnsupportedError(f"{f.get('deform')} is not a deformation framework")
    how = b.get("how")
    if b["which"] == "gimpm":
        ok = {"finite": {"undeformed", "detFij", "Fii", "Uii"},
              "infinitesimal": {"undeformed", "detΔFij", "ΔFii", "ΔUii"}}[f["deform"]]
        if how not in ok:
            # update.jl:7-28 leaves kernel2 undefined -> UndefVarError in the reference
            raise UnsupportedError(f"basis.how={how!r} is undefined for gimpm/{f['deform']}")
    cons = instr["plast"]["constitutive"]
    if cons not in CONSTITUTIVE:
        raise UnsupportedError(f"InvalidReturnMapping: {cons}")
    if cons == "MC" and dim != 2:
        raise UnsupportedError("the MC return map is plane strain only (MCRetMap.jl works on sigma[1:3])")
    if instr.get("dtype", 64) != 64:
        raise UnsupportedError("dtype=32 host arrays are not built: the C-ABI takes Float64 "
                               "arrays; use gpu.precision='mixed' for the FP32 device path")
    if instr["perf"]["status"]:
        raise UnsupportedError("perf.status=true selects the ELAST kernel, which is not built")
    for key in ("C_pf", "musl", "locking", "damping"):
        if key not in f:
            # the reference fails with a KeyError/FieldError when a partial fwrk
            # tuple drops a key that a kernel reads (kwargser.jl:36)
            raise UnsupportedError(f"fwrk.{key} is missing (top-level merge dropped it)")
    gpu = instr.get("gpu", {})
    prec = gpu.get("precision", "fp64")
    if prec not in PRECISION:
        raise UnsupportedError(f"precision {prec!r}")
    return {
        "dim": dim,
        "basis": BASIS[b["which"]],
        "how": HOW.get(how, 0) if b["which"] == "gimpm" else 0,
        "ghost": int(bool(b.get("ghost", False))),
        "deform": DEFORM[f["deform"]],
        "trsfr": TRSFR[trsfr],
        "C_pf": float(f["C_pf"]),
        "musl": int(bool(f["musl"])),
        "locking": int(bool(f["locking"])),
        "damping": float(f["damping"]),
        "constitutive": CONSTITUTIVE[cons],
        "nonloc": int(bool(instr["nonloc"]["status"])),
        "nonloc_ls": float(instr["nonloc"]["ls"]),
        "precision": PRECISION[prec],
        "jaumann": int(bool(gpu.get("jaumann", False))),
        "deterministic": int(bool(gpu.get("deterministic", False))),
    }
