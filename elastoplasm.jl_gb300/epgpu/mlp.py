"""The learned return map: a 6 -> 128 x 4 (SiLU) -> 3 network on the tensor cores.

Host wrapper of the ``epgpu_mlp_*`` functions of libepgpu.so.  The network
stands in for the 2d finite-strain Drucker-Prager return of the mixed step
(elast.jl:51-54, DP.jl:33-66) in the principal frame of the trial log strain,
scaled by the current cohesion c.  Feature rows hold 8 floats:
``[e1/s, e2/s, 0, c/2e4, tan(phi), tan(psi), phi_n, 0]`` with ``s = c/(2G)`` and
``phi_n = f_s/c`` the scaled overstress; output rows hold 4 floats, the plastic
correction per unit overstress (returned strains / s = inputs + phi_n * y).
Training runs on the GPU with the library's own forward and backward kernels.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi

NX, NY, NPARAM = abi.MLP_NX, abi.MLP_NY, abi.MLP_NPARAM
NIN, NOUT, WIDTH = 6, 3, 128
# parameter blocks of the FP32 master copy: (name, shape), W row-major (out x in)
LAYOUT = [("W1", (WIDTH, NIN)), ("b1", (WIDTH,)), ("W2", (WIDTH, WIDTH)), ("b2", (WIDTH,)),
          ("W3", (WIDTH, WIDTH)), ("b3", (WIDTH,)), ("W4", (WIDTH, WIDTH)), ("b4", (WIDTH,)),
          ("W5", (NOUT, WIDTH)), ("b5", (NOUT,))]


def _f32(a, cols):
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float32))
    if a.ndim != 2 or a.shape[1] != cols:
        raise ValueError(f"expected an (n, {cols}) float32 array, got {a.shape}")
    return a


def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def lambda_over_2G(cmpr: dict) -> float:
    """lambda / (2G) of the plane-strain stiffness (setup_cmpr.jl:21-48)."""
    D = np.asarray(cmpr["Del"], dtype=np.float64).reshape(-1)
    n = int(round(np.sqrt(D.size)))
    D = D.reshape(n, n, order="F")
    return float(D[0, 1] / (D[0, 0] - D[0, 1]))


def label(x, l2g: float) -> np.ndarray:
    """Exact FP64 labels of feature rows (library host code, the reference's DP return)."""
    lib = abi.load_library()
    x = _f32(x, NX)
    y = np.zeros((x.shape[0], NY), dtype=np.float32)
    st = lib.epgpu_mlp_label(_fp(x), x.shape[0], float(l2g), _fp(y))
    if st != abi.EP_OK:
        raise abi.EPError(st, "label")
    return y


class MLP:
    def __init__(self, seed: int = 0, l2g: float = 0.75):
        self.lib = abi.load_library()
        h = C.c_void_p()
        st = self.lib.epgpu_mlp_create(int(seed), float(l2g), C.byref(h))
        if st != abi.EP_OK:
            raise abi.EPError(st, self.lib.epgpu_last_error(None).decode())
        self.h = h
        self.l2g = l2g

    def _check(self, st):
        if st != abi.EP_OK:
            raise abi.EPError(st, self.lib.epgpu_mlp_last_error(self.h).decode())

    @property
    def params(self) -> np.ndarray:
        p = np.zeros(NPARAM, dtype=np.float32)
        self._check(self.lib.epgpu_mlp_get_params(self.h, _fp(p), NPARAM))
        return p

    @params.setter
    def params(self, p):
        p = np.ascontiguousarray(np.asarray(p, dtype=np.float32).reshape(-1))
        self._check(self.lib.epgpu_mlp_set_params(self.h, _fp(p), p.size))

    def forward(self, x) -> np.ndarray:
        x = _f32(x, NX)
        y = np.zeros((x.shape[0], NY), dtype=np.float32)
        self._check(self.lib.epgpu_mlp_forward(self.h, _fp(x), x.shape[0], _fp(y)))
        return y

    def time_forward(self, n: int, reps: int = 20) -> float:
        """Device ms of one forward launch over n rows (the kernel alone, CUDA events)."""
        ms = C.c_double(0.0)
        self._check(self.lib.epgpu_mlp_time(self.h, int(n), int(reps), C.byref(ms)))
        return ms.value

    def grad(self, x, t):
        x, t = _f32(x, NX), _f32(t, NY)
        g = np.zeros(NPARAM, dtype=np.float32)
        loss = C.c_double(0.0)
        self._check(self.lib.epgpu_mlp_grad(self.h, _fp(x), _fp(t), x.shape[0], _fp(g), C.byref(loss)))
        return g, loss.value

    def train(self, x=None, t=None, iters=100, batch=8192, lr=1e-3, seed=0) -> float:
        """Adam on mini-batches of (x, t), or of the recorded pairs when x is None."""
        loss = C.c_double(0.0)
        if x is None:
            self._check(self.lib.epgpu_mlp_train(self.h, None, None, 0, int(iters), int(batch), float(lr),
                                                 int(seed), C.byref(loss)))
        else:
            x, t = _f32(x, NX), _f32(t, NY)
            self._check(self.lib.epgpu_mlp_train(self.h, _fp(x), _fp(t), x.shape[0], int(iters), int(batch),
                                                 float(lr), int(seed), C.byref(loss)))
        return loss.value

    def record_buffer(self, capacity: int):
        self._check(self.lib.epgpu_mlp_record_buffer(self.h, int(capacity)))

    def recorded(self, copy: int = 0):
        n = C.c_int64(0)
        x = np.zeros((max(copy, 1), NX), dtype=np.float32)
        t = np.zeros((max(copy, 1), NY), dtype=np.float32)
        self._check(self.lib.epgpu_mlp_recorded(self.h, C.byref(n), _fp(x), _fp(t), int(copy)))
        k = min(n.value, copy)
        return n.value, x[:k], t[:k]

    def close(self):
        if getattr(self, "h", None):
            self.lib.epgpu_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
