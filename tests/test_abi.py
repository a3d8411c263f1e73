"""The C-ABI library: it loads and exports every symbol include/qsg.h declares.

CPU only (no kernel is launched).  The library is built here by
qusim_gb300.build (nvcc cross-compiles sm_103a without a GPU).
"""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    from qusim_gb300 import build
    path = build.build()
    from qusim_gb300 import _lib
    return _lib.load(path)


def declared_functions():
    src = open(os.path.join(ROOT, "include", "qsg.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(qsg_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_what_the_binding_lists():
    from qusim_gb300 import _lib
    assert declared_functions() == sorted(_lib.EXPORTS)


def test_library_exports_every_declared_symbol(lib):
    for name in declared_functions():
        assert hasattr(lib, name), name


def test_exports_are_plain_c_symbols():
    """No C++ mangling on the boundary: every qsg_ symbol is exported unmangled."""
    import subprocess
    from qusim_gb300 import build
    out = subprocess.run(["nm", "-D", "--defined-only", build.LIB], capture_output=True, text=True).stdout
    exported = set(l.split()[-1] for l in out.splitlines() if " T " in l)
    for name in declared_functions():
        assert name in exported, name


def test_version_and_error_without_device(lib):
    assert lib.qsg_version().startswith(b"qsg")
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present; the no-device path is not reachable")
    h = ctypes.c_void_p()
    rc = lib.qsg_init(0, 0, ctypes.byref(h))
    assert rc in (1, 3)  # no CUDA device / CUDA error, reported rather than raised
    assert lib.qsg_last_error()
    assert not h.value


def test_null_arguments_are_rejected(lib):
    assert lib.qsg_step(None, 1, 0) == 1
    assert lib.qsg_norm2(None, None) == 1
    assert lib.qsg_init(0, 0, None) == 1
    assert b"null" in lib.qsg_last_error()


def test_candidate_plans_host_only(lib):
    """Plan enumeration is host logic: every candidate has a valid geometry."""
    from qusim_gb300._lib import Plan2D
    n = lib.qsg_candidate_plans(1, 4096, 4096, None, 0)
    assert n >= 2
    arr = (Plan2D * n)()
    assert lib.qsg_candidate_plans(1, 4096, 4096, arr, n) == n
    gs = {p.g for p in arr}
    assert gs <= {1, 2, 4} and 4 in gs
    for p in arr:
        assert 4096 // p.g <= 2048
        assert p.row_e in (8, 16) and p.col_e in (8, 16, 32)
    assert lib.qsg_candidate_plans(1, 1000, 1024, None, 0) == 0
    assert lib.qsg_candidate_plans(0, 1024, 1024, None, 0) >= 1
