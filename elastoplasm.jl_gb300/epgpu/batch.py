"""Batched ensemble of independent slumps (``epgpu_batch_*`` of include/epgpu.h).

The reference runs one slump per Julia process; here n instances -- each its
own mesh, points, switches, material and time loop -- advance together: one
launch of the batch graph advances every instance by up to 16 of its own steps.
``slump_ensemble`` builds the uneven ensemble of the batched configuration:
nel_x drawn uniformly from 40..320, nel_y = nel_x / 4, 2 or 3 points per cell
and direction, friction angle uniform in 15..35 degrees, and its own seeded
exponential-covariance cohesion field per instance.
"""
from __future__ import annotations

import copy
import ctypes as C
import math

import numpy as np

from . import abi


SCHEMES = ("graphs", "persistent", "phases")


class Batch:
    def __init__(self, ics: list, instrs: list):
        self.lib = abi.load_library()
        n = len(ics)
        if n == 0 or len(instrs) != n:
            raise ValueError("one instr per instance")
        self.ics = ics
        self._cfg = (abi.ep_cfg * n)(*[abi.make_cfg(i) for i in instrs])
        self._cm = (abi.ep_cmpr * n)(*[abi.make_cmpr(ic["cmpr"]) for ic in ics])
        self._mv = [abi.MeshView(ic["mesh"]) for ic in ics]
        self._mview = (abi.ep_mesh_view * n)(*[m.view for m in self._mv])
        nmp = np.array([ic["mpts"].nmp for ic in ics], dtype=np.int64)
        h = C.c_void_p()
        st = self.lib.epgpu_batch_create(n, self._cfg, self._cm, self._mview,
                                         nmp.ctypes.data_as(C.POINTER(C.c_int64)), C.byref(h))
        if st != abi.EP_OK:
            raise abi.EPError(st, self.lib.epgpu_batch_last_error(None).decode())
        self.h = h
        self.n = n
        for i, ic in enumerate(ics):
            self._check(self.lib.epgpu_batch_upload(self.h, i, C.byref(abi.mpts_view(ic["mpts"]))))
        self.t = np.zeros(n)

    def _check(self, st):
        if st != abi.EP_OK:
            raise abi.EPError(st, self.lib.epgpu_batch_last_error(self.h).decode())

    def run(self, phase: int, T: float, tg: float = 10.0):
        """Advance every instance from its own time to T (one checkpoint window)."""
        ns = np.zeros(self.n, dtype=np.int64)
        self._check(self.lib.epgpu_batch_run(self.h, int(phase), float(T), float(tg),
                                             self.t.ctypes.data_as(C.POINTER(C.c_double)),
                                             ns.ctypes.data_as(C.POINTER(C.c_int64))))
        return self.t.copy(), ns

    def download(self, i: int):
        m = self.ics[i]["mpts"].copy()
        self._check(self.lib.epgpu_batch_download(self.h, int(i), C.byref(abi.mpts_view(m, with_topology=True))))
        return m

    def autotune(self, phase: int = 1):
        tile = C.c_int32(0)
        ms = np.zeros(3)
        self._check(self.lib.epgpu_batch_autotune(self.h, int(phase), C.byref(tile),
                                                  ms.ctypes.data_as(C.POINTER(C.c_double))))
        return tile.value, dict(zip((16, 32, 64), ms))

    def stats(self) -> dict:
        ms = C.c_double(0.0)
        nl = C.c_int64(0)
        self._check(self.lib.epgpu_batch_stats(self.h, C.byref(ms), C.byref(nl)))
        return {"device_ms": ms.value, "graph_launches": nl.value, "scheme": self.scheme()}

    def tuning(self) -> dict:
        """The autotuner's ms per batch step, per scheme and P2G tile."""
        ms = np.zeros(9)
        av = C.c_int32(0)
        self._check(self.lib.epgpu_batch_tuning(self.h, ms.ctypes.data_as(C.POINTER(C.c_double)), C.byref(av)))
        out = {name: dict(zip((16, 32, 64), ms[3 * k:3 * k + 3])) for k, name in enumerate(SCHEMES)}
        out["kernels_available"] = bool(av.value)
        return out

    def set_scheme(self, scheme: str):
        """"graphs", "persistent", "phases" or "auto" (the phase kernels when the batch qualifies)."""
        code = -1 if scheme == "auto" else SCHEMES.index(scheme)
        self._check(self.lib.epgpu_batch_set_scheme(self.h, code))

    def scheme(self) -> str:
        """The scheme the batch runs: "graphs" (the instances' own graphs), "persistent" (one
        cooperative kernel) or "phases" (one kernel per phase over all instances)."""
        return SCHEMES[self.lib.epgpu_batch_scheme(self.h)]

    def persistent(self) -> bool:
        return self.scheme() == "persistent"

    def close(self):
        if getattr(self, "h", None):
            self.lib.epgpu_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def bspline_invalid_nodes(mesh) -> int:
    """Nodes whose cubic B-spline piece the reference cannot choose, or chooses so that the basis
    loses its partition of unity.  The reference compares a node's coordinate with xB, xB + h,
    xB - h exactly (bsmpm.jl:63-76): a node that misses every comparison raises "Invalid
    position"; a node one cell inside a boundary whose rounded coordinate misses xB + h (or
    xB - h) but lies strictly inside (xB + h, xB - h) takes the interior piece instead of the
    boundary-adjacent one, the stencil weights near that boundary no longer sum to one (by 0.16),
    and the run moves without load.  Both are counted (nel_x = 320 is such a mesh)."""
    bad = 0
    for d in range(mesh.dim):
        xn = np.unique(mesh.x[d])
        x0, x1, h = float(mesh.xB[d, 0]), float(mesh.xB[d, 1]), float(mesh.h[d])
        ok = (xn == x0) | (xn == x0 + h) | (((x0 + h) < xn) & (xn < (x1 - h))) | (xn == x1 - h) | (xn == x1)
        bad += int((~ok & (xn >= x0) & (xn <= x1)).sum())
        bad += int(not np.any(xn == x0 + h)) + int(not np.any(xn == x1 - h))
    return bad


def slump_ensemble(n=256, seed=0, nelx=(40, 320), precision="mixed_df", grf=True):
    """(ics, instrs, description) of the uneven ensemble of the batched configuration.  A mesh
    whose nodes the reference's B-spline piece selection rejects or misclassifies
    (bspline_invalid_nodes) is drawn again; description[k] = (nel_x, ni, friction deg, points,
    meshes drawn again)."""
    from .ic import ic_slump
    rng = np.random.default_rng(seed)
    ics, instrs, desc = [], [], []
    fw = {"deform": "finite", "trsfr": "std", "C_pf": 1.0, "musl": True, "locking": True, "damping": 0.1}
    for k in range(n):
        redraw = 0
        while True:
            nx = int(rng.integers(nelx[0], nelx[1] + 1))
            ni = int(rng.integers(2, 4))
            phi = float(rng.uniform(15.0, 35.0))
            kw = dict(fwrk=fw, nonloc={"status": False, "ls": 0.5})
            if grf:
                kw["grf"] = {"status": True, "covariance": "exponential",
                             "param": {"Ix": [5.0, 5.0], "mean": 2.0e4, "cov": 0.3, "min": 1.0e3, "seed": 1000 + k}}
            L, nel = [64.1584, 16.0396], [nx, max(nx // 4, 1)]
            from .ic import get_geom, setup_mesh
            from .config import kwargser
            mesh = setup_mesh(kwargser(kw, dim=2), get_geom(nel, L, kwargser(kw, dim=2)))
            if bspline_invalid_nodes(mesh) == 0:
                break
            redraw += 1
        ic, cfg = ic_slump(L, nel, ni=ni, cmpr_over={"phi0": math.radians(phi)}, **kw)
        instr = copy.deepcopy(cfg["instr"])
        instr["gpu"] = {"precision": precision, "jaumann": False}
        ics.append(ic)
        instrs.append(instr)
        desc.append((nx, ni, phi, ic["mpts"].nmp, redraw))
    return ics, instrs, desc
