"""Failure paths on the host (no GPU): every bad input is an error status with a message, never a
crash, and the library keeps working afterwards (the reference's error() / SpaceMismatch /
"largest singular value is smaller than tol" conditions, src/symtensor.jl:17-28,
src/vspace.jl:8-13, src/mpsutils.jl:99-100)."""
import ctypes as C

import pytest

import mps_gb300 as mg
from mps_gb300 import _lib


def test_space_validation():
    with pytest.raises(mg.SpaceMismatch):
        mg.U1Space((0, 2), (0, 3))          # duplicate charge (vspace.jl:8-9)
    with pytest.raises(mg.SpaceMismatch):
        mg.U1Space((0, 0))                  # non-positive dimension (vspace.jl:11-13)


def test_abi_rejects_bad_arguments_with_status_and_message():
    lib = _lib.lib
    out = C.c_void_p()
    # null output pointer
    rc = lib.mpsg_meta_create(0, 1, (C.c_int32 * 1)(1), (C.c_int32 * 1)(0), (C.c_int64 * 1)(2),
                              (C.c_int32 * 1)(0), None)
    assert rc == _lib.ERR_ARGUMENT
    assert b"out" in C.string_at(lib.mpsg_last_error())
    # zero legs
    rc = lib.mpsg_meta_create(0, 0, None, None, None, None, C.byref(out))
    assert rc == _lib.ERR_ARGUMENT
    # a leg without charges
    rc = lib.mpsg_meta_create(0, 1, (C.c_int32 * 1)(0), None, None, (C.c_int32 * 1)(0),
                              C.byref(out))
    assert rc == _lib.ERR_ARGUMENT
    # the library still works
    t = mg.meta(0, (mg.U1Space((0, 2), (1, 1)), mg.U1Space((0, 2), (1, 1), isdual=True)))
    assert t.numel() == 5


def test_contract_space_mismatch_is_reported():
    V = mg.U1Space((0, 2), (1, 3))
    A = mg.meta(0, (V, V))
    with pytest.raises(mg.SpaceMismatch):   # V with V is not a dual pair
        mg.contract(A, (1, -1), A, (-1, 2))
    with pytest.raises(mg.MPSGError):       # index tuple of the wrong length
        mg.contract(A, (1, -1, 3), A, (-1, 2))


def test_truncation_below_tolerance_errors_like_the_reference():
    with pytest.raises(mg.MPSGError) as e:
        mg.truncatedsizes([[1e-3, 1e-4], [5e-4]], maxdim=4, tol=1e-2)
    assert e.value.code == _lib.ERR_TOLERANCE
    assert mg.truncatedsizes([[1.0, 1e-4], [5e-1]], maxdim=4, tol=1e-2) == [1, 1]
