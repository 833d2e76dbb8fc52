"""The C-ABI library loads and exports every symbol include/*.h declares (no GPU needed)."""
import glob
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        txt = open(h).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        names.update(re.findall(r"\b(mgt_\w+)\s*\(", txt))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "mgt_lu_factor" in names and "mgt_assemble_system" in names and len(names) >= 15


def test_library_exports_every_declared_symbol():
    from magreete_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        pytest.skip("library not built")
    lib = _lib.load()
    for name in declared_symbols():
        assert hasattr(lib, name), name
        assert name in _lib.SIGNATURES, f"{name} has no ctypes signature"
    assert lib.mgt_abi_version() == 1
    assert lib.mgt_status_string(-3).decode().startswith("singular")
