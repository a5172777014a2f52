"""The C-ABI library loads and exports every entry point include/*.h declares.

No compute call is made: this runs without a GPU.
"""
import ctypes
import glob
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    syms = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(gbfem_\w+)\s*\(", text, flags=re.M):
            syms.add(m.group(1))
    return syms


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert "gbfem_operator_apply" in syms
    assert "gbfem_dot" in syms
    assert len(syms) >= 20


def test_library_exports_every_declared_symbol(gb):
    lib = ctypes.CDLL(gb.LIB_PATH)
    missing = [s for s in sorted(declared_symbols()) if not hasattr(lib, s)]
    assert not missing, "not exported: %s" % missing


def test_version_and_error_string(gb):
    L = gb.lib()
    assert L.gbfem_version() >= 100
    assert isinstance(L.gbfem_last_error(), bytes)


def test_invalid_descriptor_is_rejected_without_gpu(gb):
    # order 9 is out of range: rejected on the host before any device call
    import pytest
    with pytest.raises(gb.GbfemError):
        gb.DGOperator((2, 2, 2), 9)
