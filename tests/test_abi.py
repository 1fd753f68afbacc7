"""The C ABI library: it loads, exports every symbol include/sw2d.h declares,
and answers host-only calls without a GPU."""
import ctypes
import os
import re

import pytest

from sw2d_efdc_gb300 import api

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    inc = os.path.join(ROOT, "include")
    for fn in os.listdir(inc):
        if not fn.endswith(".h"):
            continue
        text = open(os.path.join(inc, fn)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(sw2d_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return names


def test_library_exports_every_declared_symbol():
    lib = api.load()
    names = declared_symbols()
    assert len(names) >= 30
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing


def test_python_mirror_covers_the_header():
    assert declared_symbols() == set(api.SIGNATURES)


def test_config_default_and_abi_version():
    cfg = api.default_config()
    assert cfg.th == 1e-4 and cfg.g == 9.80 and cfg.dt == 0.04
    assert api.load().sw2d_abi_version() == 1


def test_create_rejects_bad_config_without_touching_the_gpu():
    lib = api.load()
    cfg = api.default_config(rows=1, cols=10)
    h = ctypes.c_void_p()
    assert lib.sw2d_create(ctypes.byref(cfg), ctypes.byref(h)) == -1
    assert b"rows" in lib.sw2d_last_error()
    cfg = api.default_config(rows=10, cols=10, th=0.0)
    assert lib.sw2d_create(ctypes.byref(cfg), ctypes.byref(h)) == -1


def test_status_strings():
    lib = api.load()
    assert lib.sw2d_status_string(0) == b"ok"
    assert lib.sw2d_status_string(-5) == b"HBM budget exceeded"
