"""Seeded Gaussian random fields at the material points (cohesion of the scaled-up slumps).

Host side of ``epgpu_grf_points`` (include/epgpu.h): the randomization
(spectral) method evaluated on the GPU at the point positions.  The reference's
own generator (utils/setup/mpts/GRF.jl:66-141) is a Gaussian-covariance grid
field whose exponential branch is not wired in (mpts_populate.jl:49-51); the
``instr["grf"]`` switch keeps the reference's layout (``status``,
``covariance``, ``param``), with ``param`` holding ``Ix`` (correlation lengths),
``mean``, ``cov`` (coefficient of variation), ``min`` (lower clamp), ``Nh``
(harmonics) and ``seed``.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi

COV = {"gaussian": 0, "exponential": 1}


def make_grf(dim, covariance="exponential", ell=(5.0, 5.0, 5.0), mean=2.0e4, std=6.0e3, vmin=1.0e3, nh=5000,
             seed=1234) -> abi.ep_grf:
    g = abi.ep_grf()
    g.dim = int(dim)
    g.covariance = COV[covariance]
    g.nh = int(nh)
    ell = list(ell) + [ell[-1]] * (3 - len(ell))
    for i in range(3):
        g.ell[i] = float(ell[i])
    g.mean, g.std, g.vmin, g.seed = float(mean), float(std), float(vmin), int(seed)
    return g


def spectrum(g: abi.ep_grf):
    lib = abi.load_library()
    kap = np.zeros((g.nh, g.dim))
    ab = np.zeros((g.nh, 2))
    st = lib.epgpu_grf_spectrum(C.byref(g), kap.ctypes.data_as(C.POINTER(C.c_double)),
                                ab.ctypes.data_as(C.POINTER(C.c_double)))
    if st != abi.EP_OK:
        raise abi.EPError(st, "grf spectrum")
    return kap, ab


def points(g: abi.ep_grf, X) -> np.ndarray:
    """Field values at the rows of X (n x dim) on the GPU."""
    lib = abi.load_library()
    X = np.ascontiguousarray(np.asarray(X, dtype=np.float64))
    out = np.zeros(X.shape[0])
    st = lib.epgpu_grf_points(C.byref(g), X.ctypes.data_as(C.POINTER(C.c_double)), X.shape[0],
                              out.ctypes.data_as(C.POINTER(C.c_double)))
    if st != abi.EP_OK:
        raise abi.EPError(st, lib.epgpu_last_error(None).decode())
    return out


def params(instr: dict, cmpr: dict, dim: int) -> abi.ep_grf:
    p = dict(instr["grf"].get("param", {}))
    mean = float(p.get("mean", cmpr["c0"]))
    cov = float(p.get("cov", 0.3))
    return make_grf(dim, instr["grf"].get("covariance", "gaussian"), p.get("Ix", [2.5, 2.5, 2.5])[:dim],
                    mean=mean, std=cov * mean, vmin=float(p.get("min", cmpr["cr"])), nh=int(p.get("Nh", 5000)),
                    seed=int(p.get("seed", 1234)))


def cohesion_field(X, cmpr, instr, mesh) -> np.ndarray:
    """c0 of the lattice points X (the hook of mpts_populate, mpts_populate.jl:45-51)."""
    return points(params(instr, cmpr, mesh.dim), X)
