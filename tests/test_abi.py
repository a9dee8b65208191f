"""The C-ABI library builds, loads and exports every symbol include/mara_gpu.h
declares (no compute calls: these run without a GPU)."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared(header):
    text = open(os.path.join(ROOT, "include", header)).read()
    return sorted(set(re.findall(r"\b(mara_(?:gpu|source)_\w+)\s*\(", text)))


def _declared_batch():
    text = open(os.path.join(ROOT, "include", "mara_batch.h")).read()
    return sorted(set(re.findall(r"\b(mara_batch_\w+)\s*\(", text)))


def test_header_declarations_are_bound():
    from mara2_gb300 import _native as N, batch as B
    declared = _declared("mara_gpu.h")
    assert declared, "no declarations found"
    assert sorted(N.SIGNATURES) == declared
    assert sorted(B.SIGNATURES) == _declared_batch()


def test_library_exports_every_declared_symbol():
    from mara2_gb300 import build, _native as N
    build.build()
    lib = N.load()
    for name in _declared("mara_gpu.h") + _declared_batch():
        assert hasattr(lib, name), name


def test_status_strings_without_gpu():
    from mara2_gb300 import _native as N
    assert N.status_string(N.MARA_ERR_GUARD_TOO_SMALL).startswith("Boundary region")
    assert N.status_string(0) == "success"


def test_create_rejects_bad_config_before_touching_a_device():
    import ctypes as C
    from mara2_gb300 import _native as N
    from mara2_gb300.scheme import Scheme
    cfg = N.config_from_scheme(Scheme(shape=(32, 1, 1), guard=1))
    h = C.c_void_p()
    assert N.load().mara_gpu_create(C.byref(cfg), C.byref(h)) == N.MARA_ERR_GUARD_TOO_SMALL
    cfg = N.config_from_scheme(Scheme(shape=(32, 1, 1)))
    cfg.rk_order = 4
    assert N.load().mara_gpu_create(C.byref(cfg), C.byref(h)) == N.MARA_ERR_CONFIG
