"""Python driver of the C-ABI library: one device context per (mesh, points, instr).

``Engine`` is what the reference's workflow functions would hold after
``kwargser`` built the kernel table: ``step`` replaces one MPM cycle
(workflow/worflow.jl:34-36, 80-82) and ``run`` one checkpoint window of the
time loop (worflow.jl:27-39, 73-85).  Everything goes through the exported C
functions of libepgpu.so; there is no CPU fallback: constructing an Engine
without the built library or without a GPU raises.
"""
from __future__ import annotations

import copy
import ctypes as C

import numpy as np

from . import abi


class Engine:
    def __init__(self, ic: dict, instr: dict, lib_path: str | None = None):
        self.lib = abi.load_library(lib_path)
        self.mesh = ic["mesh"]
        self.mpts = ic["mpts"]
        self.cmpr = ic["cmpr"]
        self._cfg = abi.make_cfg(instr)
        self._cm = abi.make_cmpr(self.cmpr)
        self._mv = abi.MeshView(self.mesh)
        h = C.c_void_p()
        st = self.lib.epgpu_create(C.byref(self._cfg), C.byref(self._cm), C.byref(self._mv.view),
                                   int(self.mpts.nmp), C.byref(h))
        if st != abi.EP_OK:
            raise abi.EPError(st, self.lib.epgpu_last_error(None).decode())
        self.h = h
        self.upload(self.mpts)

    # -- plumbing
    def _check(self, st: int):
        if st != abi.EP_OK:
            raise abi.EPError(st, self.lib.epgpu_last_error(self.h).decode())

    def upload(self, mpts):
        self._check(self.lib.epgpu_upload(self.h, C.byref(abi.mpts_view(mpts))))

    def fields_read(self) -> list:
        """Names of the point arrays a step of this configuration reads (``epgpu_fields_read``)."""
        return abi.names_of(self.lib.epgpu_fields_read(self.h))

    def fields_changed(self) -> list:
        """Names of the point arrays a step may change (``epgpu_fields_changed``)."""
        return abi.names_of(self.lib.epgpu_fields_changed(self.h))

    def upload_fields(self, mpts, names):
        """Upload only the named arrays; the others keep their device values (``epgpu_upload_fields``)."""
        self._check(self.lib.epgpu_upload_fields(self.h, C.byref(abi.mpts_view(mpts)), abi.mask_of(names)))

    def download_fields(self, mpts, names):
        """Download only the named arrays into ``mpts`` (``epgpu_download_fields``); vmax too."""
        self._check(self.lib.epgpu_download_fields(self.h, C.byref(abi.mpts_view(mpts)), abi.mask_of(names)))
        return mpts

    def step_fields(self, mpts, names_in, phase: int, dt: float, g, names_out=None) -> np.ndarray:
        """One host-loop step in one call (``epgpu_step_fields``): upload the named arrays of ``mpts``,
        step, download ``names_out`` (default: the same names) into ``mpts``; returns vmax."""
        g = np.zeros(3) + np.pad(np.asarray(g, dtype=np.float64), (0, 3 - len(g)))
        vmax = np.zeros(3)
        view = abi.mpts_view(mpts)
        self._check(self.lib.epgpu_step_fields(self.h, C.byref(view), abi.mask_of(names_in), int(phase), float(dt),
                                               g.ctypes.data_as(C.POINTER(C.c_double)),
                                               abi.mask_of(names_in if names_out is None else names_out),
                                               vmax.ctypes.data_as(C.POINTER(C.c_double))))
        return vmax[: self.mpts.ndim]

    def download(self, mpts=None):
        mpts = mpts or self.mpts.copy()
        self._check(self.lib.epgpu_download(self.h, C.byref(abi.mpts_view(mpts, with_topology=True))))
        return mpts

    def fields(self, names) -> dict:
        """savlot's per-point plot fields evaluated on the device (``epgpu_fields``): a dict of
        np-long FP64 arrays for the device field names of ``snapshot.FIELDS``."""
        from . import snapshot
        m = 0
        for n in names:
            if n not in snapshot.BITS:
                raise ValueError(f"UndefinedPlotOption: {n}")
            m |= snapshot.BITS[n]
        order = snapshot.rows(m)
        out = np.empty((len(order), self.mpts.nmp), dtype=np.float64)
        self._check(self.lib.epgpu_fields(self.h, m, out.ctypes.data_as(C.c_void_p)))
        return dict(zip(order, out))

    def download_mesh(self, mesh=None):
        mesh = mesh or copy.deepcopy(self.mesh)
        self._check(self.lib.epgpu_download_mesh(self.h, C.byref(abi.mesh_fields(mesh))))
        return mesh

    # -- the step
    def step(self, phase: int, dt: float, g) -> np.ndarray:
        g = np.zeros(3) + np.pad(np.asarray(g, dtype=np.float64), (0, 3 - len(g)))
        vmax = np.zeros(3)
        self._check(self.lib.epgpu_step(self.h, int(phase), float(dt), g.ctypes.data_as(C.POINTER(C.c_double)),
                                        vmax.ctypes.data_as(C.POINTER(C.c_double))))
        return vmax[: self.mpts.ndim]

    def run(self, phase: int, T: float, tg: float, t: float):
        tt = C.c_double(t)
        n = C.c_int64(0)
        self._check(self.lib.epgpu_run(self.h, int(phase), float(T), float(tg), C.byref(tt), C.byref(n)))
        return tt.value, n.value

    def run_checkpoints(self, phase: int, checks, tg: float, t: float, on_checkpoint=None):
        """One workflow phase over a checkpoint list in one call (``epgpu_run_checkpoints``): the
        library sorts the list, runs each window on the device and calls ``on_checkpoint(t, engine)``
        after it (a truthy return value stops the phase).  Returns (t, steps)."""
        arr = np.ascontiguousarray(np.asarray(checks, dtype=np.float64).ravel())
        tt = C.c_double(t)
        n = C.c_int64(0)
        failure = []

        def cb(_h, _k, t_now, _user):
            if on_checkpoint is None:
                return 0
            try:
                return 1 if on_checkpoint(t_now, self) else 0
            except BaseException as exc:          # no exception may cross the C ABI: stop and re-raise
                failure.append(exc)
                return 1

        fn = abi.CHECKPOINT_CB(cb)
        st = self.lib.epgpu_run_checkpoints(self.h, int(phase), arr.ctypes.data_as(C.POINTER(C.c_double)),
                                            int(arr.size), float(tg), C.byref(tt), fn, None, C.byref(n))
        if failure:
            raise failure[0]
        self._check(st)
        return tt.value, n.value

    def stats(self) -> dict:
        s = abi.ep_stats()
        self._check(self.lib.epgpu_stats(self.h, C.byref(s)))
        return {"steps": s.steps, "launches": s.launches, "device_ms": s.device_ms, "t": s.t,
                "plastic": s.plastic}

    def conservation(self) -> dict:
        """FP64 conservation sums of the current state (``epgpu_conservation``): point mass, momentum,
        kinetic and elastic energy, and the last step's nodal mass and momentum."""
        c = abi.ep_conservation()
        self._check(self.lib.epgpu_conservation(self.h, C.byref(c)))
        d = self.mpts.ndim
        return {"mass": c.mass, "momentum": np.array(c.momentum[:d]), "kinetic": c.kinetic,
                "elastic": c.elastic, "mass_nodes": c.mass_nodes, "momentum_nodes": np.array(c.momentum_nodes[:d])}

    def profile(self, enable: bool = True):
        self._check(self.lib.epgpu_profile(self.h, int(enable)))

    def kernel_times(self) -> dict:
        n = C.c_int32(0)
        self._check(self.lib.epgpu_profile_read(self.h, None, 0, C.byref(n)))
        arr = (abi.ep_kernel_time * max(n.value, 1))()
        self._check(self.lib.epgpu_profile_read(self.h, arr, n.value, C.byref(n)))
        return {arr[i].name.decode(): (arr[i].launches, arr[i].total_ms) for i in range(n.value)}

    def set_return_map(self, net=None, mode: str = "exact"):
        """Select the exact, learned (``net``) or recording return map (mixed 2d finite DP only)."""
        self._net = net                                   # the network must outlive its use
        self._check(self.lib.epgpu_set_return_map(self.h, net.h if net is not None else None, abi.RMAP[mode]))

    def return_map_stats(self) -> dict:
        a, b, c = C.c_int64(0), C.c_int64(0), C.c_int64(0)
        self._check(self.lib.epgpu_return_map_stats(self.h, C.byref(a), C.byref(b), C.byref(c)))
        return {"learned": a.value, "fallback": b.value, "recorded": c.value}

    def close(self):
        if getattr(self, "h", None):
            self.lib.epgpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
