"""CPU checks of the C ABI: the library loads and exports every entry point of include/mdgpu.h
(no compute call: there is no GPU here), and the ctypes mirror matches the header layout."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _header_functions():
    txt = open(os.path.join(ROOT, "include", "mdgpu.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(mdg_[a-z_0-9]+)\s*\(", txt)))


def test_library_exports_header_symbols(gpulib):
    names = _header_functions()
    assert "mdg_force_get" in names and "mdg_shake" in names and "mdg_nnlist_make" in names
    so = ctypes.CDLL(gpulib.path)
    missing = [n for n in names if not hasattr(so, n)]
    assert not missing, missing


def test_oracle_exports_same_entry_points(oracle):
    for n in _header_functions():
        base = n[len("mdg_"):]
        if base in ("create", "destroy", "last_error", "nnlist_make", "get_lists", "force_get", "shake"):
            assert oracle.has(base), n


def test_struct_sizes_match_header():
    """Compiles a probe against the header and compares struct sizes with the ctypes mirror."""
    import subprocess
    import tempfile

    from md_sim_gb300 import abi

    src = r'''
#include <stdio.h>
#include <stddef.h>
#include "mdgpu.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu\n", sizeof(mdg_sysdesc), sizeof(mdg_params), sizeof(mdg_energies),
         offsetof(mdg_sysdesc, lx), offsetof(mdg_params, shake_rptol));
  return 0;
}
'''
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "p.c")
        exe = os.path.join(d, "p")
        open(c, "w").write(src)
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), c, "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()
    got = [ctypes.sizeof(abi.SysDesc), ctypes.sizeof(abi.Params), ctypes.sizeof(abi.Energies),
           abi.SysDesc.lx.offset, abi.Params.shake_rptol.offset]
    assert [int(x) for x in out] == got


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    import md_sim_gb300

    monkeypatch.setattr(md_sim_gb300, "LIBPATH", str(tmp_path / "nope.so"))
    monkeypatch.setattr(md_sim_gb300, "_lib", None)
    with pytest.raises(RuntimeError):
        md_sim_gb300.load()
