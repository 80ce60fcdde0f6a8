"""The C-ABI library builds for sm_103a, loads, and exports every function
that include/epgpu.h declares (no compute call: no GPU needed)."""
import ctypes as C
import os
import re

from conftest import ROOT


def declared_functions():
    src = open(os.path.join(ROOT, "include", "epgpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(epgpu_\w+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    from epgpu import abi
    from epgpu.build import build
    path = build()
    lib = C.CDLL(path)
    names = declared_functions()
    assert len(names) >= 11
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # the ctypes signature table covers the header
    assert set(names) <= set(abi.SIGNATURES), set(names) - set(abi.SIGNATURES)


def test_version_string_without_gpu():
    from epgpu import abi
    lib = abi.load_library()
    assert b"sm_103a" in lib.epgpu_version()


def test_create_rejects_bad_arguments_without_gpu():
    # argument validation happens before any CUDA call
    from epgpu import abi, ic_slump
    lib = abi.load_library()
    ic, cfg = ic_slump([64.1584, 16.0396], [40, 10])
    c = abi.make_cfg(cfg["instr"])
    c.trsfr = 7
    h = C.c_void_p()
    mv = abi.MeshView(ic["mesh"])
    st = lib.epgpu_create(C.byref(c), C.byref(abi.make_cmpr(ic["cmpr"])), C.byref(mv.view), ic["mpts"].nmp,
                          C.byref(h))
    assert st == 2 and b"transfer" in lib.epgpu_last_error(None)
    assert lib.epgpu_destroy(None) == 1


def test_batch_rejects_bad_arguments_without_gpu():
    import ctypes as C
    from epgpu import abi
    lib = abi.load_library()
    h = C.c_void_p()
    assert lib.epgpu_batch_create(0, None, None, None, None, C.byref(h)) == 1
    assert lib.epgpu_batch_destroy(None) == 1
    assert lib.epgpu_batch_instance(None, 0) is None
