"""The C-ABI library builds, loads and exports every entry point that
include/om_gb300.h declares (no compute calls: no GPU needed)."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", fn)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names |= set(re.findall(r"\b(om_[a-z0-9_]+)\s*\(", txt))
    return names


def test_header_symbols_exported(om_lib):
    lib = om_lib.load_library()
    names = declared_symbols()
    assert len(names) >= 20
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing
    assert set(om_lib.EXPORTS) <= names


def test_version_and_defaults(om_lib):
    lib = om_lib.load_library()
    assert b"sm_103a" in lib.om_version()
    cfg = om_lib.default_config()
    assert cfg.boundary == 0 and cfg.precision == 32 and abs(cfg.gamma - 5 / 3) < 1e-15
    assert cfg.use_graph == 1


def test_create_without_gpu_fails_cleanly(om_lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(om_lib.OMError) as e:
        om_lib.Life((16, 16))
    assert e.value.status in (1, 2)


def test_bad_arguments_rejected(om_lib):
    lib = om_lib.load_library()
    import ctypes as C
    h = C.c_void_p()
    sizes = (C.c_int * 2)(0, 5)
    assert lib.om_create(1, 2, sizes, None, C.byref(h)) == 1
    assert b"sizes" in lib.om_last_error()
    assert lib.om_create(9, 2, sizes, None, C.byref(h)) == 1
    assert lib.om_destroy(None) == 0
