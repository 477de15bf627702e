"""The C-ABI library builds, loads and exports every entry declared in include/mw_gb300.h (no GPU needed)."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_entries():
    src = open(os.path.join(ROOT, "include", "mw_gb300.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char \*)\s*(mw_\w+)\(", src, re.M)))


def test_header_declares_the_boundary():
    names = declared_entries()
    for must in ("mw_ctx_create", "mw_apply", "mw_apply_batch", "mw_multiply", "mw_add", "mw_op_create_poisson",
                 "mw_op_create_helmholtz", "mw_tree_upload", "mw_tree_download", "mw_last_error"):
        assert must in names


def test_library_exports_every_declared_symbol(engine):
    import ctypes
    lib = ctypes.CDLL(engine.LIB_PATH)
    missing = [n for n in declared_entries() if not hasattr(lib, n)]
    assert not missing, missing
    assert set(engine.EXPORTS) == set(declared_entries())


def test_bad_arguments_rejected_without_device(engine):
    import ctypes
    lib = engine.load_library()
    h = ctypes.c_void_p()
    corner = (ctypes.c_int * 3)(-1, -1, -1)
    boxes = (ctypes.c_int * 3)(2, 2, 2)
    # order out of range is rejected before any CUDA call
    assert lib.mw_ctx_create(0, -5, corner, boxes, 42, 1, 25, ctypes.byref(h)) == 1
    assert b"order" in lib.mw_last_error(None)
    assert lib.mw_apply(1e-3, None, None, None, 0, None, -1, 0, 0) == 1


def test_no_host_fallback_without_gpu(engine):
    """Without a usable device the engine fails loudly instead of computing on the host."""
    if engine.cuda_available():
        pytest.skip("a CUDA device is present")
    with pytest.raises(engine.MWError):
        engine.MultiResolutionAnalysis(5)
