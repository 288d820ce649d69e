"""The C-ABI library loads and exports every entry point of include/mpgpu.h
(no device call: runs without a GPU)."""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "mpgpu.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    names = set(re.findall(r"\b((?:mpgpu|mpgen)_[a-z_0-9]+)\s*\(", txt))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_symbols()
    for n in ("mpgpu_create", "mpgpu_loopbf", "mpgpu_solve", "mpgpu_avprod", "mpgpu_mupdat"):
        assert n in names


def test_library_exports_all_declared(mp):
    lib = mp.lib()
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_export_list_matches_header(mp):
    assert sorted(set(mp.EXPORTS)) == declared_symbols()
