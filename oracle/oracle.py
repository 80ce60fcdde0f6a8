"""ctypes driver of the FP64 CPU oracle (oracle/eporacle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke`` as
the checker and by ``bench.py`` for the CPU baseline.  The product never
imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libeporacle.so")
PROBE = os.path.join(HERE, "_build", "libscalarprobe.so")   # the library's scalar header, for tests


def build(force: bool = False) -> str:
    srcs = [os.path.join(HERE, f) for f in ("eporacle.cpp", "eporacle.h", "scalar_probe.cpp", "Makefile")]
    srcs.append(os.path.join(HERE, "..", "elastoplasm.jl_gb300", "csrc", "ep_scalar.h"))
    outs = (LIB, PROBE)
    if force or not all(os.path.exists(o) for o in outs) or any(
            os.path.getmtime(s) > min(os.path.getmtime(o) for o in outs) for s in srcs):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        from epgpu import abi
        build()
        L = C.CDLL(LIB)
        P = C.POINTER
        L.eporacle_create.restype = C.c_void_p
        L.eporacle_create.argtypes = [P(abi.ep_cfg), P(abi.ep_cmpr), P(abi.ep_mesh_view), C.c_int64]
        L.eporacle_upload.argtypes = [C.c_void_p, P(abi.ep_mpts_view)]
        L.eporacle_step.argtypes = [C.c_void_p, C.c_int32, C.c_double, P(C.c_double), P(C.c_double)]
        L.eporacle_run.argtypes = [C.c_void_p, C.c_int32, C.c_double, C.c_double, P(C.c_double), P(C.c_int64)]
        L.eporacle_download.argtypes = [C.c_void_p, P(abi.ep_mpts_view)]
        L.eporacle_download_mesh.argtypes = [C.c_void_p, P(abi.ep_mesh_fields)]
        L.eporacle_e2n.argtypes = [C.c_void_p, P(C.c_int64)]
        L.eporacle_set_threads.argtypes = [C.c_void_p, C.c_int]
        L.eporacle_set_threads.restype = None
        L.eporacle_last_error.restype = C.c_char_p
        L.eporacle_last_error.argtypes = [C.c_void_p]
        L.eporacle_destroy.argtypes = [C.c_void_p]
        L.eporacle_destroy.restype = None
        _lib = L
    return _lib


class Oracle:
    """Serial FP64 MPM step on the host, same interface as :class:`epgpu.Engine`."""

    def __init__(self, ic: dict, instr: dict, threads: int = 1):
        from epgpu import abi
        self.abi = abi
        self.ic = ic
        self.mesh = ic["mesh"]
        self.mpts = ic["mpts"]
        self._cfg = abi.make_cfg(instr)
        self._cmpr = abi.make_cmpr(ic["cmpr"])
        self._mv = abi.MeshView(self.mesh)
        L = lib()
        self.h = L.eporacle_create(C.byref(self._cfg), C.byref(self._cmpr), C.byref(self._mv.view),
                                   int(self.mpts.nmp))
        if not self.h:
            raise RuntimeError("eporacle_create failed")
        L.eporacle_set_threads(self.h, int(threads))
        self._check(L.eporacle_upload(self.h, C.byref(abi.mpts_view(self.mpts))))

    def _check(self, st):
        if st != 0:
            raise self.abi.EPError(st, lib().eporacle_last_error(self.h).decode())

    def step(self, phase: int, dt: float, g) -> np.ndarray:
        g = np.asarray(g, dtype=np.float64)
        vmax = np.zeros(3)
        self._check(lib().eporacle_step(self.h, int(phase), float(dt), g.ctypes.data_as(C.POINTER(C.c_double)),
                                        vmax.ctypes.data_as(C.POINTER(C.c_double))))
        return vmax[: self.mpts.ndim]

    def run(self, phase: int, T: float, tg: float, t: float):
        tt = C.c_double(t)
        n = C.c_int64(0)
        self._check(lib().eporacle_run(self.h, int(phase), float(T), float(tg), C.byref(tt), C.byref(n)))
        return tt.value, n.value

    def download(self, mpts=None):
        mpts = mpts or self.mpts.copy()
        self._check(lib().eporacle_download(self.h, C.byref(self.abi.mpts_view(mpts, with_topology=True))))
        return mpts

    def fields(self, names) -> dict:
        """savlot's plot fields (device names of epgpu.snapshot.FIELDS) from the downloaded state,
        by the restatement of plot.jl in plot_oracle.py: the checker of Engine.fields."""
        import plot_oracle as po
        m = self.download()
        x, z = po.plot_coords(m)
        out = {}
        for n in names:
            out[n] = x.copy() if n == "x" else z.copy() if n == "z" else po.plot_field(m, n)
        return out

    def download_mesh(self, mesh=None):
        import copy
        mesh = mesh or copy.deepcopy(self.mesh)
        self._check(lib().eporacle_download_mesh(self.h, C.byref(self.abi.mesh_fields(mesh))))
        return mesh

    def e2n(self):
        out = np.zeros_like(self.mesh.e2n, order="F")
        self._check(lib().eporacle_e2n(self.h, out.ctypes.data_as(C.POINTER(C.c_int64))))
        return out

    def close(self):
        if self.h:
            lib().eporacle_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
