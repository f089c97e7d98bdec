"""The C-ABI library builds for sm_103a, loads on a host without a GPU, exports every symbol the
header declares, and its table structs match the host planner's numpy dtypes. No compute calls."""
import os
import re

import pytest

from conftest import ROOT


def _declared():
    src = open(os.path.join(ROOT, "include", "tnkit_gb300.h")).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\*?\s+(tnk_\w+)\s*\(", src, re.M)))


def test_library_builds_and_exports_every_declared_symbol():
    from tnkit_gb300 import build, _lib
    path = build.build()
    assert os.path.exists(path)
    lib = _lib.load(path)
    decl = _declared()
    assert decl and set(decl) == set(_lib.exported_symbols())
    for name in decl:
        assert hasattr(lib, name), name
    assert b"sm_103a" in lib.tnk_version()


def test_struct_layouts_match_planner_dtypes():
    from tnkit_gb300 import _lib
    import ctypes as C
    lib = _lib.load()
    sizes = (C.c_int64 * 6)()
    assert lib.tnk_struct_sizes(C.cast(sizes, C.c_void_p)) == 0
    assert list(sizes) == [32, 56, 16, 32, 24, 16]
    assert [d.itemsize for d in (_lib.GEMM_TASK, _lib.GEMM_SEG, _lib.GEMM_TILE, _lib.COMB_TASK,
                                 _lib.COMB_TERM, _lib.COMB_ITEM)] == list(sizes)
    assert C.sizeof(_lib.Plan3) == 19 * 8


def test_null_plan_is_an_error_not_a_crash():
    """Argument validation happens on the host before any launch."""
    from tnkit_gb300 import _lib
    lib = _lib.load()
    rc = lib.tnk_contract3_f64(None, None, None, None, None, None, 0, None)
    assert rc == _lib.TNK_ERR_ARG
    assert b"null plan" in lib.tnk_last_error()
