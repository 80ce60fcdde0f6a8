"""Build recipe of libepgpu.so (the C-ABI library) for sm_103a with nvcc.

Each translation unit compiles in parallel; the FP64 step is compiled with
``-fmad=false`` so that no multiply-add is contracted (its results must match
an unfused host computation bit for bit).  Output: ``lib/libepgpu.so`` next to
this package (in-tree, git-ignored).
"""
from __future__ import annotations

import os
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "lib")
REPO = os.path.dirname(PKG)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
          "--expt-relaxed-constexpr", "-I", os.path.join(REPO, "include")]
UNITS = {
    "ep_api.cu": [],
    "ep_sort.cu": [],
    "ep_fp64.cu": ["-fmad=false"],
    "ep_mixed.cu": [],
    "ep_mlp.cu": [],
    "ep_grf.cu": [],
}


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.sep not in c or os.path.exists(c)):
            return c
    return "nvcc"


def _compile(unit: str, extra: list[str], verbose: bool) -> str:
    src = os.path.join(CSRC, unit)
    obj = os.path.join(LIBDIR, unit.replace(".cu", ".o"))
    cmd = [nvcc(), *ARCH, *COMMON, *extra, "-c", src, "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {unit}:\n{r.stderr}")
    if verbose:
        print(r.stderr)
    return obj


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(LIBDIR, exist_ok=True)
    out = os.path.join(LIBDIR, "libepgpu.so")
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(REPO, "include", "epgpu.h")]
    if not force and os.path.exists(out) and all(os.path.getmtime(d) <= os.path.getmtime(out) for d in deps):
        return out
    with ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(lambda kv: _compile(kv[0], kv[1], verbose), UNITS.items()))
    cmd = [nvcc(), *ARCH, "-shared", "-o", out, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    return out


if __name__ == "__main__":
    import sys
    print(build(force=True, verbose="-v" in sys.argv))
