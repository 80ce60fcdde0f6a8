"""The allocation-free binning entry point, for callers that cannot allocate.

Some callers of this library must not allocate device memory while they call
it -- e.g. a Julia or PyTorch host whose caching allocator owns the device's
memory budget, or a pipeline in which cudaMalloc/cudaFree would stall other
streams.  ``epgpu_bin_cells_noalloc`` serves them: it keeps its scratch in a
static device array instead of allocating.  This test calls it through the C
ABI twice in a row, on two different point clouds (so scratch left over from
the first call would show up in the second), and checks each result against
the allocating ``epgpu_bin_cells`` on the same input.  Binning is integer
work, so the tolerance is zero: outputs must be identical.  It also checks the
rejection of a mesh larger than the static scratch.

This file is collected last on purpose (name order).
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bin(lib, fn, mesh, x_dev, n, torch):
    nc = int(np.prod(mesh.nel[: mesh.dim]))
    p2e = torch.full((n,), -7, dtype=torch.int32, device="cuda")
    start = torch.full((nc + 1,), -7, dtype=torch.int32, device="cuda")
    lst = torch.full((n,), -7, dtype=torch.int32, device="cuda")
    nel = (C.c_int64 * 3)(*mesh.nel[: mesh.dim], *([0] * (3 - mesh.dim)))
    h = (C.c_double * 3)(*mesh.h, *([0.0] * (3 - mesh.dim)))
    x0 = (C.c_double * 3)(*mesh.x0, *([0.0] * (3 - mesh.dim)))
    st = getattr(lib, fn)(mesh.dim, nel, h, x0, C.c_void_p(x_dev.data_ptr()), n, C.c_void_p(p2e.data_ptr()),
                          C.c_void_p(start.data_ptr()), C.c_void_p(lst.data_ptr()), None)
    assert st == 0, (fn, st)
    torch.cuda.synchronize()
    return p2e.cpu().numpy(), start.cpu().numpy(), lst.cpu().numpy()


def test_noalloc_binning_matches_allocating_entry_point():
    import torch
    from epgpu import abi, ic_slump
    lib = abi.load_library()
    # the 2d slump at nel=[640,160]: 102,400 cells, 365,024 points
    ic, _ = ic_slump([64.1584, 16.0396], [640, 160], ni=3)
    mesh, pts = ic["mesh"], ic["mpts"]
    n = pts.nmp
    rng = np.random.default_rng(11)
    clouds = [pts.x + rng.normal(scale=0.2, size=pts.x.shape),
              pts.x[:, ::-1] + rng.normal(scale=1.5, size=pts.x.shape)]   # different cells, some outside
    for x in clouds:
        xd = torch.tensor(np.ascontiguousarray(x), dtype=torch.float64, device="cuda")
        ref = _bin(lib, "epgpu_bin_cells", mesh, xd, n, torch)
        got = _bin(lib, "epgpu_bin_cells_noalloc", mesh, xd, n, torch)
        for a, b in zip(got, ref):
            assert np.array_equal(a, b)
        assert ref[1][-1] == n and np.all(np.diff(ref[1]) >= 0)


def test_noalloc_rejects_meshes_beyond_its_scratch():
    import torch
    from epgpu import abi
    lib = abi.load_library()
    nel = (C.c_int64 * 3)(1024, 1024, 0)           # 1,048,576 cells > EPGPU_NOALLOC_MAX_CELLS
    h = (C.c_double * 3)(1.0, 1.0, 0.0)
    x0 = (C.c_double * 3)(0.0, 0.0, 0.0)
    x = torch.zeros(2 * 4, dtype=torch.float64, device="cuda")
    out = torch.zeros(4 * 3 + 1024 * 1024 + 1, dtype=torch.int32, device="cuda")
    st = lib.epgpu_bin_cells_noalloc(2, nel, h, x0, C.c_void_p(x.data_ptr()), 4, C.c_void_p(out.data_ptr()),
                                     C.c_void_p(out.data_ptr() + 16), C.c_void_p(out.data_ptr() + 32), None)
    assert st == 1
    assert b"524288" in lib.epgpu_last_error(None)
