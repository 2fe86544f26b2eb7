"""GB300-native force / neighbour-list / SHAKE hot path for md_sim (vlcekl/md_sim).

The CUDA library (md_sim_gb300/_build/libmdgpu.so, C ABI in include/mdgpu.h) replaces the
reference's force_get, nnlist_make and move_shake.  `load()` returns the bound library and fails
loudly when it has not been built: there is no CPU fallback.
"""
import os

from .abi import Context, Lib, MdgError, RunParams  # noqa: F401

HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(HERE, "_build", "libmdgpu.so")

_lib = None


def load() -> Lib:
    global _lib
    if _lib is None:
        if not os.path.exists(LIBPATH):
            raise RuntimeError(f"{LIBPATH} is missing: run md_sim_gb300/build.py (or __graft_entry__.build())")
        _lib = Lib(LIBPATH, "mdg_")
    return _lib
