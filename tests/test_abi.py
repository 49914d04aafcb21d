"""CPU-only checks of the C ABI library: it builds, loads, exports every
symbol declared in include/subby_gb300.h, and rejects bad inputs on the host
before touching a GPU (no compute calls here)."""
import ctypes as ct
import os
import re

import numpy as np
import pytest

from subby_gb300 import _lib

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))


def _declared():
    with open(os.path.join(ROOT, "include", "subby_gb300.h")) as f:
        src = f.read()
    return sorted(set(re.findall(r"\b(subby_[a-z_0-9]+)\s*\(", src)))


def test_header_and_binding_agree():
    assert sorted(_lib.EXPORTS) == _declared()


def test_library_loads_and_exports_every_symbol():
    lib = _lib.load()
    for name in _declared():
        assert hasattr(lib, name), name
    assert b"sm_103a" in lib.subby_version()
    assert lib.subby_strerror(_lib.ERR_TREE) == b"invalid tree"


def _create(parent, A=4):
    lib = _lib.load()
    R = len(parent)
    parent = np.ascontiguousarray(parent, dtype=np.int32)
    dist = np.full(R, 0.1)
    ev = np.zeros(A)
    V = np.eye(A)
    pi = np.full(A, 1.0 / A)
    h = ct.c_void_p()
    p = lambda a: a.ctypes.data_as(ct.c_void_p)  # noqa: E731
    rc = lib.subby_plan_create(p(parent), p(dist), p(ev), p(V), p(pi), R, A, ct.byref(h))
    return rc, lib.subby_last_error().decode()


@pytest.mark.parametrize("parent,msg", [
    ([-1, 0, 0, 0], "has 3 children"),
    ([-1, 0], "has 1 children"),
    ([0, 0, 0], "must be negative"),
    ([-1, 2, 0], "is not in"),
    ([-1, 0, 0, 1], "has 1 children"),
])
def test_invalid_trees_rejected_on_host(parent, msg):
    rc, err = _create(parent)
    assert rc == _lib.ERR_TREE
    assert msg in err


def test_unsupported_alphabet_rejected():
    rc, err = _create([-1, 0, 0], A=100)
    assert rc == _lib.ERR_UNSUPPORTED


def test_null_arguments_rejected():
    lib = _lib.load()
    assert lib.subby_plan_create(None, None, None, None, None, 3, 4, None) == _lib.ERR_ARG
    assert lib.subby_plan_run(None, None, 0, None, None, None, 0, 0, None, 0, None) == _lib.ERR_ARG
