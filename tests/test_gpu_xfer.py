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


@pytest.mark.parametrize("precision", ["fp64", "mixed", "mixed_df"])
@pytest.mark.parametrize("pinned", [False, True])
@pytest.mark.parametrize("trsfr", ["std", "tpic"])
def test_masked_transfers_continue_the_run(precision, trsfr, pinned):
    """A host loop that moves only the state a step reads and changes (epgpu_upload_fields /
    epgpu_download_fields with epgpu_fields_read & epgpu_fields_changed) after a full first upload
    gives the run that keeps the state on the device; the constants are not moved again.  Bit for bit
    for the FP64 step and for the mixed step with FP64 accumulators; with double-float accumulators a
    few points differ by the last bit of the 48-bit pair (1.8e-15 relative in F and b_e after one step),
    which can flip the last bit of an FP32 stress later, so that case is held to FP32 resolution
    (1e-7 of each field's scale).  With page-locked host arrays the mixed precisions take the direct
    transfers (one pass between the host arrays and the step's layout, no FP64 staging), held to the
    same run."""
    from epgpu import Engine, ic_slump
    fw = {"deform": "finite", "trsfr": trsfr, "C_pf": 0.99, "musl": True, "locking": True, "damping": 0.1}
    ic, cfg = ic_slump(*C1, fwrk=fw, nonloc={"status": False, "ls": 0.5})
    instr = copy.deepcopy(cfg["instr"])
    instr["gpu"] = {"precision": precision, "jaumann": False, "deterministic": precision != "fp64"}
    g = [0.0, -9.81]
    ref = Engine(copy.deepcopy(ic), instr)
    for k in range(6):
        ref.step(1, 0.02, g)
    want = ref.download()
    ref.close()
    e = Engine(copy.deepcopy(ic), instr)
    moved = sorted(set(e.fields_read()) & set(e.fields_changed()))
    assert {"x", "v", "Fij", "bij", "tau", "epII", "dlam"} <= set(moved)
    assert not {"c0", "cr", "phi", "Omega0", "u", "p"} & set(moved)
    keep = []
    host = _pinned(ic["mpts"], keep) if pinned else ic["mpts"].copy()
    for k in range(6):
        e.upload_fields(host, moved)
        e.step(1, 0.02, g)
        e.download_fields(host, moved)
    for f in moved:
        a, b = np.asarray(getattr(host, f)), np.asarray(getattr(want, f))
        if precision == "mixed_df":
            assert np.abs(a - b).max() <= 1e-7 * max(np.abs(b).max(), 1e-300), f
        else:
            assert np.array_equal(a, b), f
    e.close()


def test_masked_upload_needs_every_field_read_once():
    import ctypes as C
    from epgpu import Engine, abi, ic_slump
    from epgpu.abi import EPError
    ic, cfg = ic_slump(*C1, nonloc={"status": False, "ls": 0.5})
    lib = abi.load_library()
    # a fresh context: a masked upload that leaves out fields the step reads is refused, naming them
    c, cm, mv = abi.make_cfg(cfg["instr"]), abi.make_cmpr(ic["cmpr"]), abi.MeshView(ic["mesh"])
    h = C.c_void_p()
    assert lib.epgpu_create(C.byref(c), C.byref(cm), C.byref(mv.view), ic["mpts"].nmp, C.byref(h)) == 0
    view = abi.mpts_view(ic["mpts"])
    assert lib.epgpu_upload_fields(h, C.byref(view), abi.mask_of(["x", "v"])) == 1
    msg = lib.epgpu_last_error(h).decode()
    assert "never uploaded" in msg and "Fij" in msg and "c0" in msg
    assert lib.epgpu_upload_fields(h, C.byref(view), lib.epgpu_fields_read(h)) == 0
    assert lib.epgpu_upload_fields(h, C.byref(view), abi.mask_of(["x", "v"])) == 0
    lib.epgpu_destroy(h)
    # a field named in the mask must be given
    e = Engine(copy.deepcopy(ic), cfg["instr"])
    m = ic["mpts"].copy()
    m.v = None
    with pytest.raises(EPError) as ex:
        e.upload_fields(m, ["x", "v"])
    assert ex.value.status == 1 and "NULL: v" in str(ex.value)
    e.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed_df"])
def test_masked_download_writes_only_the_mask(precision):
    from epgpu import Engine, ic_slump
    ic, cfg = ic_slump(*C1, nonloc={"status": False, "ls": 0.5})
    instr = copy.deepcopy(cfg["instr"])
    if precision != "fp64":
        instr["gpu"] = {"precision": precision, "jaumann": False}
    e = Engine(copy.deepcopy(ic), instr)
    e.step(1, 0.02, [0.0, -9.81])
    full = e.download()
    host = ic["mpts"].copy()
    for f in _fields(host):
        getattr(host, f)[...] = np.nan
    e.download_fields(host, ["x", "tau"])
    assert np.array_equal(host.x, full.x) and np.array_equal(host.tau, full.tau)
    assert np.isnan(host.v).all() and np.isnan(host.eij).all()
    e.close()


@pytest.mark.parametrize("dim,precision", [(2, "mixed"), (2, "mixed_df"), (3, "mixed_df")])
def test_direct_and_staged_masked_transfers_agree(dim, precision):
    """The mixed precisions' masked transfers of page-locked host arrays (direct: the host arrays to and
    from the step's layout in one pass) and of pageable ones (through the FP64 staging layout) leave the
    same bits, on the host after every download and in the run's end state."""
    from epgpu import Engine, ic_slump
    L, nel = C1 if dim == 2 else C1_3D
    ic, cfg = ic_slump(L, nel, nonloc={"status": False, "ls": 0.5})
    instr = copy.deepcopy(cfg["instr"])
    instr["gpu"] = {"precision": precision, "jaumann": False, "deterministic": True}
    g = [0.0] * (dim - 1) + [-9.81]
    runs = {}
    for pinned in (False, True):
        keep = []
        e = Engine(copy.deepcopy(ic), instr)
        moved = sorted(set(e.fields_read()) & set(e.fields_changed()))
        host = _pinned(ic["mpts"], keep) if pinned else ic["mpts"].copy()
        seen = []
        for k in range(5):
            e.upload_fields(host, moved)
            e.step(1, 0.02, g)
            e.download_fields(host, moved)
            seen.append({f: np.array(getattr(host, f)) for f in moved})
        runs[pinned] = (seen, e.download())
        e.close()
    (sa, fa), (sb, fb) = runs[False], runs[True]
    for k in range(len(sa)):
        for f in sa[k]:
            assert np.array_equal(sa[k][f], sb[k][f]), (k, f)
    for f in ("x", "v", "tau", "Fij", "bij", "epII", "dlam", "sig", "J"):
        assert np.array_equal(np.asarray(getattr(fa, f)), np.asarray(getattr(fb, f))), f


@pytest.mark.parametrize("pinned", [False, True])
@pytest.mark.parametrize("precision", ["fp64", "mixed_df"])
def test_step_fields_equals_the_three_calls(precision, pinned):
    """epgpu_step_fields (upload, step, download in one call: for mapped page-locked arrays in the
    mixed precisions on the device with one synchronisation, part of the arrays moving on a second
    stream beside the step) against epgpu_upload_fields + epgpu_step + epgpu_download_fields: the same
    bits on the host and the same vmax after every step.  The host changes the moved arrays between
    steps, so that a step reading an array before its upload landed, or a download taken before the
    step wrote it, shows."""
    from epgpu import Engine, ic_slump
    ic, cfg = ic_slump(*C1, nonloc={"status": False, "ls": 0.5})
    instr = copy.deepcopy(cfg["instr"])
    instr["gpu"] = {"precision": precision, "jaumann": False, "deterministic": precision != "fp64"}
    g = [0.0, -9.81]
    out = []
    for fused in (False, True):
        keep = []
        e = Engine(copy.deepcopy(ic), instr)
        moved = sorted(set(e.fields_read()) & set(e.fields_changed()))
        host = _pinned(ic["mpts"], keep) if pinned else ic["mpts"].copy()
        vs, seen = [], []
        for k in range(5):
            if fused:
                vm = e.step_fields(host, moved, 1, 0.02, g)
            else:
                e.upload_fields(host, moved)
                vm = e.step(1, 0.02, g)
                e.download_fields(host, moved)
            vs.append(np.array(vm))
            seen.append({f: np.array(getattr(host, f)) for f in moved})
            # a host loop's own change of the state before the next step
            getattr(host, "Fij")[...] *= 1.0 + 1e-4
            getattr(host, "epII")[...] += 1e-6
            getattr(host, "v")[...] *= 0.999
            getattr(host, "x")[...] += 1e-5
        assert e.stats()["steps"] == 5
        out.append((vs, seen))
        e.close()
    (va, sa), (vb, sb) = out
    for k in range(len(va)):
        assert np.array_equal(va[k], vb[k]), k
        for f in sa[k]:
            assert np.array_equal(sa[k][f], sb[k][f]), (k, f)
