"""Point-state transfers through the C ABI (epgpu_upload / epgpu_download).

Host buffers that the runtime reports as page-locked and mapped are read and written in place by
one transfer kernel (k_xfer, which also transposes AoS <-> SoA); pageable buffers go through the
copy engine and the staging area.  Both routes must leave the same bits on the device and on the
host, for every field, in 2d and 3d, FP64 and the mixed precisions.
"""
import copy

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

C1 = ([64.1584, 64.1584 / 4.0], [40, 10])
C1_3D = ([64.1584, 16.0396, 16.0396], [16, 4, 4])


def _fields(mpts):
    return [k for k, v in mpts.__dict__.items() if isinstance(v, np.ndarray) and v.dtype == np.float64]


def _pinned(mpts, keep):
    """The same state in page-locked host memory (pinned tensors viewed as numpy arrays)."""
    torch = pytest.importorskip("torch")
    q = mpts.copy()
    for k in _fields(q):
        v = getattr(q, k)
        t = torch.from_numpy(np.ascontiguousarray(v.reshape(-1, order="F"))).pin_memory()
        keep.append(t)
        setattr(q, k, t.numpy().reshape(v.shape, order="F"))
    return q


def _nan_filled(mpts, pinned, keep):
    q = _pinned(mpts, keep) if pinned else mpts.copy()
    for k in _fields(q):
        getattr(q, k)[...] = np.nan
    return q


@pytest.mark.parametrize("dim,precision", [(2, "fp64"), (2, "mixed_df"), (3, "fp64"), (3, "mixed")])
def test_pinned_and_pageable_transfers_agree(dim, precision):
    from epgpu import Engine, ic_slump
    L, nel = C1 if dim == 2 else C1_3D
    ic, cfg = ic_slump(L, nel, nonloc={"status": False, "ls": 0.5})
    instr = copy.deepcopy(cfg["instr"])
    # the deterministic mode makes the mixed steps of the two engines comparable bit for bit
    instr["gpu"] = {"precision": precision, "jaumann": False, "deterministic": precision != "fp64"}
    g = [0.0] * (dim - 1) + [-9.81]
    keep = []
    got = {}
    for pinned in (False, True):
        e = Engine(copy.deepcopy(ic), instr)
        src = _pinned(ic["mpts"], keep) if pinned else ic["mpts"].copy()
        e.upload(src)
        first = e.download(_nan_filled(ic["mpts"], pinned, keep))   # round trip of the uploaded state
        for _ in range(3):
            e.step(1, 0.01, g)
        after = e.download(_nan_filled(ic["mpts"], pinned, keep))
        e.close()
        got[pinned] = (first, after)
    for i, what in enumerate(("round trip", "after 3 steps")):
        a, b = got[False][i], got[True][i]
        for k in _fields(a):
            assert np.array_equal(getattr(a, k), getattr(b, k), equal_nan=True), f"{what}: {k}"
    # the FP64 round trip returns the state that was uploaded (ϕ is read on upload only, for its
    # tan/sin/cos; the mixed layout stores positions as cell + FP32 offset)
    if precision == "fp64":
        a = got[True][0]
        for k in ("x", "v", "tau", "sig", "Fij", "bij", "c0", "l"):
            assert np.array_equal(getattr(a, k), getattr(ic["mpts"], k)), k
