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
    # APIC in the mixed precisions on a mesh where the reference's D⁻¹ could differ from I (h = 4.01)
    ic, cfg = ic_slump([64.1584, 16.0396], [16, 4])
    c = abi.make_cfg(cfg["instr"])
    c.trsfr, c.precision = 2, 1
    mv = abi.MeshView(ic["mesh"])
    st = lib.epgpu_create(C.byref(c), C.byref(abi.make_cmpr(ic["cmpr"])), C.byref(mv.view), ic["mpts"].nmp,
                          C.byref(h))
    assert st == 2 and b"apic" in lib.epgpu_last_error(None) and not h.value
    # the device-field call checks its handle before anything else
    assert lib.epgpu_fields(None, 1, None) == 1


def test_batch_rejects_bad_arguments_without_gpu():
    import ctypes as C
    from epgpu import abi
    lib = abi.load_library()
    h = C.c_void_p()
    assert lib.epgpu_batch_create(0, None, None, None, None, C.byref(h)) == 1
    assert lib.epgpu_batch_destroy(None) == 1
    assert lib.epgpu_batch_instance(None, 0) is None


def test_struct_layouts_match_the_header(tmp_path):
    """The ctypes mirror of every struct (epgpu/abi.py, which the Julia binding copies field by field)
    has the header's size and field offsets, as gcc lays them out."""
    import shutil
    import subprocess
    import pytest
    from epgpu import abi
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("gcc not found")
    structs = [abi.ep_cfg, abi.ep_cmpr, abi.ep_mesh_view, abi.ep_mesh_fields, abi.ep_mpts_view, abi.ep_grf,
               abi.ep_kernel_time, abi.ep_stats, abi.ep_conservation]
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "epgpu.h"', "int main(void) {"]
    for S in structs:
        n = S.__name__
        lines.append(f'    printf("{n} sizeof %zu\\n", sizeof({n}));')
        for f, _ in S._fields_:
            lines.append(f'    printf("{n} {f} %zu\\n", offsetof({n}, {f}));')
    lines += ["    return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([gcc, "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {tuple(l.split()[:2]): int(l.split()[2]) for l in out if l.strip()}
    bad = []
    for S in structs:
        n = S.__name__
        if got[(n, "sizeof")] != C.sizeof(S):
            bad.append((n, "sizeof", got[(n, "sizeof")], C.sizeof(S)))
        for f, _ in S._fields_:
            off = getattr(S, f).offset
            if got[(n, f)] != off:
                bad.append((n, f, got[(n, f)], off))
    assert not bad, bad


def test_field_mask_bits_match_the_header():
    """EP_MPTS_* of include/epgpu.h against the Python mirror (epgpu/abi.py MPTS_BITS), which follows
    the order of the ep_mpts_view arrays."""
    from epgpu import abi
    src = open(os.path.join(ROOT, "include", "epgpu.h")).read()
    bits = {n: 1 << int(k) for n, k in re.findall(r"#define EP_MPTS_(\w+)\s+\(1ull << (\d+)\)", src)}
    names = {"X": "x", "L0": "l0", "L": "l", "N0": "n0", "N": "n", "OMEGA0": "Omega0", "OMEGA": "Omega",
             "DJ": "dJ", "J": "J", "U": "u", "V": "v", "P": "p", "RHO0": "rho0", "RHO": "rho", "C0": "c0",
             "CR": "cr", "PHI": "phi", "DLAM": "dlam", "EPII": "epII", "EPV": "epV", "SIG": "sig", "TAU": "tau",
             "DVIJ": "dvij", "DUIJ": "duij", "DFIJ": "dFij", "FIJ": "Fij", "BIJ": "bij", "EIJ": "eij", "WIJ": "wij",
             "SJIJ": "sJij", "APIC_B": "Bij", "APIC_D": "Dij"}
    assert len(bits) == 32
    assert {names[k]: v for k, v in bits.items()} == abi.MPTS_BITS
    fields = [f for f, _ in abi.ep_mpts_view._fields_ if f not in ("ndim", "nmp", "vmax", "p2e", "p2n")]
    assert fields == list(abi.MPTS_BITS)


def test_julia_binding_mirrors_the_ctypes_structs():
    """The Julia extension (julia/GB300Ext.jl) declares each ABI struct with the ctypes mirror's fields
    in the same order and of the same C width (Julia is absent here, so the layout is checked as text
    against the ctypes mirror, which test_struct_layouts_match_the_header holds to gcc's layout)."""
    import ctypes as C
    from epgpu import abi
    src = open(os.path.join(ROOT, "elastoplasm.jl_gb300", "julia", "GB300Ext.jl")).read()
    width = {"Int32": 4, "Int64": 8, "Float64": 8, "Ptr{Float64}": 8, "Ptr{UInt8}": 8, "Ptr{Int64}": 8}
    pairs = {"EpCfg": abi.ep_cfg, "EpCmpr": abi.ep_cmpr, "EpMeshView": abi.ep_mesh_view, "EpMptsView": abi.ep_mpts_view}
    for jl, S in pairs.items():
        body = re.search(rf"struct {jl}\n(.*?)\nend", src, re.S).group(1)
        decl = []
        for name, typ in re.findall(r"(\w+)::([\w{},]+)", body):
            m = re.match(r"NTuple\{(\d+),(\w+)\}", typ)
            decl.append((name, int(m.group(1)) * width[m.group(2)] if m else width[typ]))
        ours = [(f, C.sizeof(t)) for f, t in S._fields_]
        assert decl == ours, (jl, decl, ours)
