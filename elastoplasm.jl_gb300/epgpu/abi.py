"""ctypes mirror of include/epgpu.h and views of the set-up arrays.

The structures below match the C declarations field by field; the helpers
build them from the :class:`epgpu.ic.Mesh` / :class:`epgpu.ic.Point` arrays,
which already have the reference's column-major layout, so no copy is made on
the host side.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .config import to_abi

_D = C.POINTER(C.c_double)
_F = C.POINTER(C.c_float)
_I64 = C.POINTER(C.c_int64)

EP_OK = 0
STATUS = {0: "EP_OK", 1: "EP_ERR_ARG", 2: "EP_ERR_UNSUPPORTED", 3: "EP_ERR_NONFINITE",
          5: "EP_ERR_TIMEOUT", 6: "EP_ERR_CUDA", 7: "EP_ERR_INVALID_POSITION",
          8: "EP_ERR_NOMEM", 9: "EP_ERR_STATE", 10: "EP_ERR_NONCONVERGED"}


class ep_cfg(C.Structure):
    _fields_ = [("dim", C.c_int32), ("basis", C.c_int32), ("how", C.c_int32), ("ghost", C.c_int32),
                ("deform", C.c_int32), ("trsfr", C.c_int32), ("C_pf", C.c_double), ("musl", C.c_int32),
                ("locking", C.c_int32), ("damping", C.c_double), ("constitutive", C.c_int32),
                ("nonloc", C.c_int32), ("nonloc_ls", C.c_double), ("precision", C.c_int32),
                ("jaumann", C.c_int32), ("deterministic", C.c_int32)]


class ep_cmpr(C.Structure):
    _fields_ = [("E", C.c_double), ("nu", C.c_double), ("Kc", C.c_double), ("Gc", C.c_double),
                ("Del", C.c_double * 36), ("Hp", C.c_double), ("c0", C.c_double), ("cr", C.c_double),
                ("phi0", C.c_double), ("phir", C.c_double), ("rho0", C.c_double), ("c", C.c_double)]


class ep_mesh_view(C.Structure):
    _fields_ = [("dim", C.c_int64), ("nel", C.c_int64 * 4), ("nno", C.c_int64 * 4), ("nn", C.c_int64),
                ("h", C.c_double * 3), ("x0", C.c_double * 3), ("x", _D), ("xB", _D),
                ("bcs", C.POINTER(C.c_uint8)), ("e2n", _I64)]


class ep_mesh_fields(C.Structure):
    _fields_ = [("mi", _D), ("p", _D), ("v", _D), ("a", _D), ("oobf", _D), ("dJ", _D)]


_MPTS_FIELDS = ["vmax", "x", "l0", "l", "n0", "n", "Omega0", "Omega", "dJ", "J", "u", "v", "p",
                "rho0", "rho", "c0", "cr", "phi", "dlam", "epII", "epV", "sig", "tau",
                "dvij", "duij", "dFij", "Fij", "bij", "eij", "wij", "sJij"]


# EP_MPTS_* bits of include/epgpu.h: one per array of ep_mpts_view, in this order
MPTS_BITS = {f: 1 << k for k, f in enumerate(["x", "l0", "l", "n0", "n", "Omega0", "Omega", "dJ", "J", "u", "v", "p",
                                              "rho0", "rho", "c0", "cr", "phi", "dlam", "epII", "epV", "sig", "tau",
                                              "dvij", "duij", "dFij", "Fij", "bij", "eij", "wij", "sJij", "Bij",
                                              "Dij"])}


def mask_of(names) -> int:
    m = 0
    for n in names:
        m |= MPTS_BITS[n]
    return m


def names_of(mask: int) -> list:
    return [f for f, b in MPTS_BITS.items() if mask & b]


class ep_mpts_view(C.Structure):
    _fields_ = ([("ndim", C.c_int64), ("nmp", C.c_int64)] + [(f, _D) for f in _MPTS_FIELDS]
                + [("p2e", _I64), ("p2n", _I64), ("Bij", _D), ("Dij", _D)])


class ep_grf(C.Structure):
    _fields_ = [("dim", C.c_int32), ("covariance", C.c_int32), ("nh", C.c_int32), ("pad_", C.c_int32),
                ("ell", C.c_double * 3), ("mean", C.c_double), ("std", C.c_double), ("vmin", C.c_double),
                ("seed", C.c_uint64)]


class ep_kernel_time(C.Structure):
    _fields_ = [("name", C.c_char * 32), ("launches", C.c_int64), ("total_ms", C.c_double)]


class ep_stats(C.Structure):
    _fields_ = [("steps", C.c_int64), ("launches", C.c_int64), ("device_ms", C.c_double),
                ("t", C.c_double), ("plastic", C.c_int64)]


class ep_conservation(C.Structure):
    _fields_ = [("mass", C.c_double), ("momentum", C.c_double * 3), ("kinetic", C.c_double),
                ("elastic", C.c_double), ("mass_nodes", C.c_double), ("momentum_nodes", C.c_double * 3)]


def _dptr(a: np.ndarray):
    assert a.dtype == np.float64 and (a.flags.f_contiguous or a.flags.c_contiguous)
    return a.ctypes.data_as(_D)


def make_cfg(instr: dict) -> ep_cfg:
    f = to_abi(instr)
    return ep_cfg(**f)


def make_cmpr(cmpr: dict) -> ep_cmpr:
    c = ep_cmpr()
    for k in ("E", "nu", "Kc", "Gc", "Hp", "c0", "cr", "phi0", "phir", "rho0", "c"):
        setattr(c, k, float(cmpr[k]))
    D = np.asarray(cmpr["Del"], dtype=np.float64)
    flat = D.flatten(order="F")
    for i, v in enumerate(flat):
        c.Del[i] = float(v)
    return c


class MeshView:
    """Holds an ``ep_mesh_view`` plus references to the arrays it points to."""

    def __init__(self, mesh):
        d = mesh.dim
        v = ep_mesh_view()
        v.dim = d
        for i in range(d + 1):
            v.nel[i] = int(mesh.nel[i])
            v.nno[i] = int(mesh.nno[i])
        v.nn = int(mesh.nn)
        for i in range(d):
            v.h[i] = float(mesh.h[i])
            v.x0[i] = float(mesh.x0[i])
        self._x = np.asfortranarray(mesh.x, dtype=np.float64)
        self._xB = np.asfortranarray(mesh.xB, dtype=np.float64)
        self._bcs = np.asfortranarray(mesh.bcs.astype(np.uint8))
        self._e2n = np.asfortranarray(mesh.e2n, dtype=np.int64)
        v.x = _dptr(self._x)
        v.xB = _dptr(self._xB)
        v.bcs = self._bcs.ctypes.data_as(C.POINTER(C.c_uint8))
        v.e2n = self._e2n.ctypes.data_as(_I64)
        self.view = v


def mpts_view(mpts, with_topology: bool = False) -> ep_mpts_view:
    """View of every array of a :class:`Point` (arrays must stay alive)."""
    v = ep_mpts_view()
    v.ndim = mpts.ndim
    v.nmp = mpts.nmp
    for f in _MPTS_FIELDS:
        a = getattr(mpts, f)
        if a is not None:                        # None: a NULL pointer (skipped or refused by the call)
            setattr(v, f, _dptr(a))
    if with_topology and mpts.p2e is not None:
        v.p2e = mpts.p2e.ctypes.data_as(_I64)
        v.p2n = mpts.p2n.ctypes.data_as(_I64)
    for f in ("Bij", "Dij"):                     # APIC state (types.jl:82-83)
        a = getattr(mpts, f, None)
        if a is not None:
            setattr(v, f, _dptr(a))
    return v


def mesh_fields(mesh) -> ep_mesh_fields:
    f = ep_mesh_fields()
    f.mi = _dptr(mesh.mi)
    f.p = _dptr(mesh.p)
    f.v = _dptr(mesh.v)
    f.a = _dptr(mesh.a)
    f.oobf = _dptr(mesh.oobf)
    # mesh.ΔJ is dim x nno but only its first nno linear slots are used (volumetric.jl:8)
    f.dJ = _dptr(mesh.dJ)
    return f


def library_path() -> str:
    here = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    return os.path.join(here, "lib", "libepgpu.so")


# ep_checkpoint_cb: int32_t (*)(ep_handle* h, int32_t k, double t, void* user)
CHECKPOINT_CB = C.CFUNCTYPE(C.c_int32, C.c_void_p, C.c_int32, C.c_double, C.c_void_p)

# exported C symbols and their ctypes signatures (kept in step with include/epgpu.h)
SIGNATURES = {
    "epgpu_version": (C.c_char_p, []),
    "epgpu_create": (C.c_int, [C.POINTER(ep_cfg), C.POINTER(ep_cmpr), C.POINTER(ep_mesh_view), C.c_int64,
                               C.POINTER(C.c_void_p)]),
    "epgpu_upload": (C.c_int, [C.c_void_p, C.POINTER(ep_mpts_view)]),
    "epgpu_step": (C.c_int, [C.c_void_p, C.c_int32, C.c_double, _D, _D]),
    "epgpu_run": (C.c_int, [C.c_void_p, C.c_int32, C.c_double, C.c_double, _D, _I64]),
    "epgpu_run_checkpoints": (C.c_int, [C.c_void_p, C.c_int32, _D, C.c_int32, C.c_double, _D, CHECKPOINT_CB,
                                        C.c_void_p, _I64]),
    "epgpu_download": (C.c_int, [C.c_void_p, C.POINTER(ep_mpts_view)]),
    "epgpu_upload_fields": (C.c_int, [C.c_void_p, C.POINTER(ep_mpts_view), C.c_uint64]),
    "epgpu_download_fields": (C.c_int, [C.c_void_p, C.POINTER(ep_mpts_view), C.c_uint64]),
    "epgpu_step_fields": (C.c_int, [C.c_void_p, C.POINTER(ep_mpts_view), C.c_uint64, C.c_int32, C.c_double, _D,
                                    C.c_uint64, _D]),
    "epgpu_fields_read": (C.c_uint64, [C.c_void_p]),
    "epgpu_fields_changed": (C.c_uint64, [C.c_void_p]),
    "epgpu_download_mesh": (C.c_int, [C.c_void_p, C.POINTER(ep_mesh_fields)]),
    "epgpu_fields": (C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p]),
    "epgpu_stats": (C.c_int, [C.c_void_p, C.POINTER(ep_stats)]),
    "epgpu_conservation": (C.c_int, [C.c_void_p, C.POINTER(ep_conservation)]),
    "epgpu_destroy": (C.c_int, [C.c_void_p]),
    "epgpu_profile": (C.c_int, [C.c_void_p, C.c_int32]),
    "epgpu_profile_read": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.POINTER(C.c_int32)]),
    "epgpu_last_error": (C.c_char_p, [C.c_void_p]),
    "epgpu_bin_cells": (C.c_int, [C.c_int32, _I64, _D, _D, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p,
                                  C.c_void_p, C.c_void_p]),
    "epgpu_bin_cells_noalloc": (C.c_int, [C.c_int32, _I64, _D, _D, C.c_void_p, C.c_int64, C.c_void_p,
                                          C.c_void_p, C.c_void_p, C.c_void_p]),
    # learned return map
    "epgpu_mlp_create": (C.c_int, [C.c_uint64, C.c_double, C.POINTER(C.c_void_p)]),
    "epgpu_mlp_destroy": (C.c_int, [C.c_void_p]),
    "epgpu_mlp_last_error": (C.c_char_p, [C.c_void_p]),
    "epgpu_mlp_set_params": (C.c_int, [C.c_void_p, _F, C.c_int64]),
    "epgpu_mlp_get_params": (C.c_int, [C.c_void_p, _F, C.c_int64]),
    "epgpu_mlp_forward": (C.c_int, [C.c_void_p, _F, C.c_int64, _F]),
    "epgpu_mlp_time": (C.c_int, [C.c_void_p, C.c_int64, C.c_int32, C.POINTER(C.c_double)]),
    "epgpu_mlp_grad": (C.c_int, [C.c_void_p, _F, _F, C.c_int64, _F, _D]),
    "epgpu_mlp_train": (C.c_int, [C.c_void_p, _F, _F, C.c_int64, C.c_int32, C.c_int32, C.c_float, C.c_uint64,
                                  _D]),
    "epgpu_mlp_label": (C.c_int, [_F, C.c_int64, C.c_double, _F]),
    "epgpu_mlp_record_buffer": (C.c_int, [C.c_void_p, C.c_int64]),
    "epgpu_mlp_recorded": (C.c_int, [C.c_void_p, _I64, _F, _F, C.c_int64]),
    "epgpu_set_return_map": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32]),
    "epgpu_selftest_wait_timeout": (C.c_int, [C.c_int64]),
    "epgpu_batch_create": (C.c_int, [C.c_int32, C.POINTER(ep_cfg), C.POINTER(ep_cmpr), C.POINTER(ep_mesh_view),
                                     _I64, C.POINTER(C.c_void_p)]),
    "epgpu_batch_upload": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(ep_mpts_view)]),
    "epgpu_batch_download": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(ep_mpts_view)]),
    "epgpu_batch_run": (C.c_int, [C.c_void_p, C.c_int32, C.c_double, C.c_double, _D, _I64]),
    "epgpu_batch_autotune": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_int32), _D]),
    "epgpu_batch_stats": (C.c_int, [C.c_void_p, _D, _I64]),
    "epgpu_batch_scheme": (C.c_int32, [C.c_void_p]),
    "epgpu_batch_tuning": (C.c_int, [C.c_void_p, _D, C.POINTER(C.c_int32)]),
    "epgpu_batch_set_scheme": (C.c_int, [C.c_void_p, C.c_int32]),
    "epgpu_batch_instance": (C.c_void_p, [C.c_void_p, C.c_int32]),
    "epgpu_batch_last_error": (C.c_char_p, [C.c_void_p]),
    "epgpu_batch_destroy": (C.c_int, [C.c_void_p]),
    "epgpu_grf_spectrum": (C.c_int, [C.POINTER(ep_grf), _D, _D]),
    "epgpu_grf_points": (C.c_int, [C.POINTER(ep_grf), _D, C.c_int64, _D]),
    "epgpu_return_map_stats": (C.c_int, [C.c_void_p, _I64, _I64, _I64]),
}

# learned return map constants (include/epgpu.h)
MLP_NX, MLP_NY, MLP_NPARAM = 8, 4, 50819
RMAP = {"exact": 0, "learned": 1, "record": 2}

_lib = None


def load_library(path: str | None = None):
    """Load libepgpu.so (fails loudly when it was not built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or library_path()
    if not os.path.exists(p):
        raise RuntimeError(f"libepgpu.so not built ({p}); run __graft_entry__.build()")
    lib = C.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


class EPError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status
