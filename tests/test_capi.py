"""The C ABI without a GPU: the library loads and exports every symbol
include/*.h declares; status strings; invalid arguments are rejected before any
device work; workspace queries and tuning keys are host-only."""
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


def _lib_or_skip():
    from magreete_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        pytest.skip("library not built")
    return _lib, _lib.load()


def test_status_strings():
    L, lib = _lib_or_skip()
    codes = [L.MGT_OK, L.MGT_ERR_ARG, L.MGT_ERR_CUDA, L.MGT_ERR_SINGULAR, L.MGT_ERR_TIMEOUT,
             L.MGT_ERR_WORKSPACE, L.MGT_ERR_UNSUPPORTED, L.MGT_ERR_NOT_CONVERGED]
    texts = [lib.mgt_status_string(c).decode() for c in codes]
    assert all(texts) and len(set(texts)) == len(texts)
    assert lib.mgt_status_string(-99).decode()


def test_invalid_arguments_rejected_before_any_device_work():
    """Null pointers, non-positive sizes, short leading dimensions and unknown
    kinds / dtypes return MGT_ERR_ARG (the checks precede every CUDA call)."""
    import ctypes
    L, lib = _lib_or_skip()
    ARG = L.MGT_ERR_ARG
    nb = ctypes.c_size_t()
    null = None
    assert lib.mgt_lu_workspace_bytes(L.MGT_C128, 0, ctypes.byref(nb)) == ARG
    assert lib.mgt_lu_workspace_bytes(7, 100, ctypes.byref(nb)) == ARG
    assert lib.mgt_lu_workspace_bytes(L.MGT_C64, 100, None) == ARG
    assert lib.mgt_lu_solve_workspace_bytes(L.MGT_C64, 100, 0, ctypes.byref(nb)) == ARG
    assert lib.mgt_residual_workspace_bytes(0, 4, ctypes.byref(nb)) == ARG
    assert lib.mgt_refine_workspace_bytes(100, 0, ctypes.byref(nb)) == ARG
    assert lib.mgt_propagate_workspace_bytes(9, 10, 10, 1, ctypes.byref(nb)) == ARG
    assert lib.mgt_cgemm_workspace_bytes(0, ctypes.byref(nb)) == ARG
    assert lib.mgt_lu_factor(L.MGT_C64, null, 100, 100, null, null, 0, null) == ARG
    assert lib.mgt_lu_factor_static(L.MGT_C64, null, 100, 100, null, null, null) == ARG
    assert lib.mgt_lu_solve(L.MGT_C64, null, 100, 100, null, null, 4, null, 4, 4, null, 0, null) == ARG
    assert lib.mgt_residual(null, 100, 100, null, 4, null, 4, null, 4, 4, null, 0, null) == ARG
    assert lib.mgt_residual_prepare(null, 100, 100, null, 0, null) == ARG
    assert lib.mgt_residual_apply(100, null, 4, null, 4, null, 4, 4, null, 0, null) == ARG
    assert lib.mgt_solve_refined(null, 100, null, 100, null, 100, null, 4, null, 4, 4, 1e-10, 10, null, 0,
                                 None, None, null) == ARG
    assert lib.mgt_refine_start(null, 100, null, 100, null, 4, null, 4, 4, null, 0, null) == ARG
    assert lib.mgt_refine_prepare(null, 100, 100, 4, null, 0, null) == ARG
    assert lib.mgt_refine_correct(null, 100, null, 100, null, 100, null, 4, null, 4, 4, null, 0, null) == ARG
    assert lib.mgt_refine_norms(null, 100, 100, null, 4, null, 4, 4, null, 0, null, null) == ARG
    assert lib.mgt_column_dots(null, 4, null, 4, 100, 4, null, null) == ARG
    assert lib.mgt_cgemm_sub(L.MGT_C64, 1, 0, 4, 4, null, 4, null, 4, null, 4, null, 0, null) == ARG
    assert lib.mgt_assemble_system(99, null, 10, 1.0, 0.0, 0.0, 0.0, 0.0, null, 10, L.MGT_C128, null, 0, 0,
                                   null) == ARG
    assert lib.mgt_assemble_propagator(L.MGT_2D_VECTOR, null, 10, null, 10, 1.0, 1.0, 0.0, 0, 0.0, 0, 0.0, 0.0,
                                       0, null, 10, null) == ARG
    assert lib.mgt_workspace_status(null, None, null) == ARG


def test_workspace_queries_are_host_only_and_grow_with_size():
    import ctypes
    L, lib = _lib_or_skip()

    def q(fn, *args):
        nb = ctypes.c_size_t()
        L.check(fn(*args, ctypes.byref(nb)))
        return nb.value

    for dt in (L.MGT_C128, L.MGT_C64):
        small, big = q(lib.mgt_lu_workspace_bytes, dt, 500), q(lib.mgt_lu_workspace_bytes, dt, 20000)
        assert 0 < small <= big
        assert q(lib.mgt_lu_solve_workspace_bytes, dt, 500, 8) <= q(lib.mgt_lu_solve_workspace_bytes, dt, 5000, 64)
    # the residual needs at least the double-float copy of X (16 B per entry)
    assert q(lib.mgt_residual_workspace_bytes, 1000, 16) >= 1000 * 16 * 16
    assert q(lib.mgt_refine_workspace_bytes, 1000, 16) >= 1000 * 16 * 16
    assert q(lib.mgt_propagate_workspace_bytes, L.MGT_3D_VECTOR, 100, 1000, 8) > 0


def test_tuning_keys_round_trip_and_range_checks():
    L, lib = _lib_or_skip()
    keys = {L.MGT_TUNE_PANEL_ROWS: (128, [16, 5000]), L.MGT_TUNE_OUTER_BLOCK: (64, [32, 256]),
            L.MGT_TUNE_PANEL_MAX_CTAS: (40, [-1]), L.MGT_TUNE_PANEL_REGISTERS: (2, [3, -1]),
            L.MGT_TUNE_TC_PRECISION: (L.MGT_TC_TF32X3, [5]), L.MGT_TUNE_COOPERATIVE: (0, []),
            L.MGT_TUNE_LOOKAHEAD: (0, []), L.MGT_TUNE_FUSED_RIGHT: (0, []), L.MGT_TUNE_PANEL_CLUSTER: (0, []),
            L.MGT_TUNE_SYM_ASSEMBLY: (0, []), L.MGT_TUNE_WIDE_UPDATE: (4096, [-1])}
    saved = {k: lib.mgt_get_tuning(k) for k in keys}
    try:
        for k, (good, bad) in keys.items():
            assert lib.mgt_set_tuning(k, good) == L.MGT_OK and lib.mgt_get_tuning(k) == good
            for v in bad:
                assert lib.mgt_set_tuning(k, v) == L.MGT_ERR_ARG and lib.mgt_get_tuning(k) == good
        assert lib.mgt_set_tuning(999, 1) == L.MGT_ERR_ARG and lib.mgt_get_tuning(999) == L.MGT_ERR_ARG
    finally:
        for k, v in saved.items():
            lib.mgt_set_tuning(k, v)
    assert {k: lib.mgt_get_tuning(k) for k in keys} == saved


def test_python_constants_match_the_header():
    """Every #define MGT_* of the header has the same value in _lib.py, and
    every tuning key is documented in INTEGRATION.md."""
    from magreete_gb300 import _lib
    defines = {}
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        for name, val in re.findall(r"#define\s+(MGT_\w+)\s+\(?(-?\d+)\)?", open(h).read()):
            defines[name] = int(val)
    assert len(defines) >= 25
    for name, val in defines.items():
        assert hasattr(_lib, name), name
        assert getattr(_lib, name) == val, name
    doc = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    for name in defines:
        if name.startswith("MGT_TUNE_"):
            assert name in doc, f"{name} missing from INTEGRATION.md"
