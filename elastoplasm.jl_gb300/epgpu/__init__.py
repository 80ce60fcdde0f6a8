"""epgpu: GB300-native explicit MPM step for ElastoPlasm.jl (host side).

The compute path is the C-ABI library ``lib/libepgpu.so`` (include/epgpu.h),
hand-written CUDA for sm_103a.  This package mirrors the reference's host
interface around it: ``ic_slump``/``ic_collapse`` (set-up), ``slump``/``slump_``
/``collapse``/``elastoplasm`` (workflow) and ``require``/``kwargser`` (switches).
"""
from .config import kwargser, require
from .ic import ic_collapse, ic_slump
from .workflow import collapse, elastoplasm, slump, slump_

__all__ = ["require", "kwargser", "ic_slump", "ic_collapse", "slump", "slump_", "collapse", "elastoplasm",
           "Engine"]


def __getattr__(name):
    if name == "Engine":
        from .engine import Engine
        return Engine
    raise AttributeError(name)
