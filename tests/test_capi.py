"""The C ABI library: loads without a GPU, exports every entry point the
headers declare, and rejects misuse without touching a device."""
import ctypes as C
import os
import re

import pytest

from amat_gb300 import _native

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared(header):
    src = open(os.path.join(ROOT, "include", header)).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(afm_[a-z0-9_]+)\s*\(", src)))


@pytest.mark.parametrize("header,loader,sigs", [
    ("afm.h", _native.libafm, _native.AFM_SIGNATURES),
    ("afm_problems.h", _native.libproblems, _native.PROBLEM_SIGNATURES),
])
def test_every_declared_symbol_is_exported(header, loader, sigs):
    lib = loader()
    names = declared(header)
    assert names, header
    for n in names:
        assert hasattr(lib, n), n
        assert n in sigs, "binding missing for " + n


def test_status_strings():
    lib = _native.libafm()
    for code, name in _native.STATUS.items():
        assert lib.afm_status_string(code).decode() == name
    assert lib.afm_status_string(999).decode() == "UNKNOWN_STATUS"


def test_null_operator_is_rejected():
    lib = _native.libafm()
    assert lib.afm_finalize(None) == 105
    assert lib.afm_matvec(None, None, None, 1) == 105
    assert b"null" in lib.afm_last_error()
    assert lib.afm_destroy(None) == 0


def test_create_validates_arguments():
    lib = _native.libafm()
    h = C.c_void_p()
    assert lib.afm_create(None, 0, 0) == 105
    assert lib.afm_create(C.byref(h), 7, 0) == 10  # UNKNOWN_BC_METH


def test_server_calls_reject_null_handles():
    """The serving calls check their handle before touching a device."""
    lib = _native.libafm()
    info = (C.c_uint64 * 6)()
    assert lib.afm_server_set_lane(None, 1 << 20, 32) == 105
    assert lib.afm_server_set_inner_format(None, 4) == 105
    assert lib.afm_server_set_priorities(None, 1) == 105
    assert lib.afm_server_get_info(None, info) == 105
    assert lib.afm_server_poll(None, None, None) == 105
    assert lib.afm_server_destroy(None) == 0
    assert lib.afm_server_create(None, 0, 0, 0) == 105
    assert lib.afm_set_fused_colours(None, 1) == 105
    assert lib.afm_matvec_inner_device(None, None, None, None) == 105
