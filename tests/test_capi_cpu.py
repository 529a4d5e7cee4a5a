"""CPU-only checks of the C ABI library: it loads and exports every symbol
include/simit_gb300.h declares (no compute calls without a GPU)."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = []
    for f in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if f.endswith(".h"):
            src = open(os.path.join(ROOT, "include", f)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names += re.findall(r"^\s*(?:int|void\s*\*|const char\s*\*)\s*(sg_\w+)\s*\(", src,
                                flags=re.M)
    return sorted(set(names))


def test_library_exports_every_declared_symbol():
    from simit_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        from simit_gb300 import build
        build.build()
    import ctypes
    L = ctypes.CDLL(_lib.LIB_PATH)
    decl = _declared()
    assert len(decl) >= 10
    missing = [n for n in decl if not hasattr(L, n)]
    assert not missing, missing
    # every declared symbol has a ctypes signature in the binding
    assert not [n for n in decl if n not in _lib.SIGNATURES]


def test_loading_without_gpu_reports_cleanly():
    """sg_ctx_create fails with an error code (no exception, no crash) when no
    device is visible."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    from simit_gb300 import _lib
    import ctypes
    h = ctypes.c_void_p()
    rc = _lib.load().sg_ctx_create(0, ctypes.byref(h))
    assert rc != 0
    assert _lib.load().sg_last_error()
