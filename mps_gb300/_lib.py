"""ctypes binding of ``libmpsgb300.so`` (declarations in ``include/mpsgb300.h``).

The library is built in-tree by ``mps_gb300.build``; it is loaded from this directory only, and
importing fails loudly when it cannot be built or loaded: there is no fallback path.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

_HERE = os.path.dirname(os.path.abspath(__file__))

OK = 0
ERR_ARGUMENT = 1
ERR_SPACE_MISMATCH = 2
ERR_CUDA = 3
ERR_NO_CONVERGENCE = 4
ERR_UNSUPPORTED = 5
ERR_TOLERANCE = 6


class MPSGError(RuntimeError):
    """Failure reported by the C ABI; ``code`` is the MPSG_ERR_* status."""

    def __init__(self, code, msg):
        super().__init__(f"[mpsg status {code}] {msg}")
        self.code = code


class SpaceMismatch(MPSGError):
    """The reference's SpaceMismatch / SectorMismatch / error() on incompatible spaces."""


class NoConvergence(MPSGError):
    pass


_ERRORS = {ERR_SPACE_MISMATCH: SpaceMismatch, ERR_NO_CONVERGENCE: NoConvergence}

P = C.c_void_p
I32 = C.c_int32
I64 = C.c_int64
F64 = C.c_double
PI32 = C.POINTER(C.c_int32)
PI64 = C.POINTER(C.c_int64)
PF64 = C.POINTER(C.c_double)
PP = C.POINTER(C.c_void_p)

# name -> argtypes (every function returns int status)
SIGNATURES = {
    "mpsg_version": [],
    "mpsg_ctx_create": [C.c_int, PP],
    "mpsg_ctx_destroy": [P],
    "mpsg_ctx_synchronize": [P],
    "mpsg_ctx_counters": [P, PI64, PF64],
    "mpsg_ctx_clear_caches": [P],
    "mpsg_ctx_stream": [P, PP],
    "mpsg_ctx_set_timing": [P, I32],
    "mpsg_ctx_kernel_time": [P, I32, PF64, PI64, PF64],
    "mpsg_tensor_create": [P, I32, I32, PI32, PI32, PI64, PI32, PP],
    "mpsg_tensor_free": [P],
    "mpsg_tensor_rank": [P, PI32],
    "mpsg_tensor_charge": [P, PI32],
    "mpsg_tensor_numel": [P, PI64, PI64],
    "mpsg_tensor_is_diagonal": [P, PI32],
    "mpsg_tensor_space": [P, I32, PI32, PI32, PI64, PI32],
    "mpsg_tensor_sectors": [P, PI32, PI64, PI64],
    "mpsg_tensor_upload": [P, PF64, I64],
    "mpsg_tensor_download": [P, PF64, I64],
    "mpsg_tensor_device_ptr": [P, PP],
    "mpsg_device_checks": [P, I32, PI64, PI64],
    "mpsg_host_alloc": [I64, PP],
    "mpsg_host_free": [P],
    "mpsg_tensor_download_async": [P, P, P, I64, PP],
    "mpsg_tensor_upload_async": [P, P, P, I64, PP],
    "mpsg_copy_wait": [P, P],
    "mpsg_copy_query": [P, PI32],
    "mpsg_copy_synchronize": [P],
    "mpsg_copy_free": [P],
    "mpsg_tensor_copy": [P, P, PP],
    "mpsg_dual": [P, P, PP],
    "mpsg_permutelegs": [P, P, PI32, PP],
    "mpsg_fuselegs": [P, P, I32, I32, I32, PP],
    "mpsg_splitleg": [P, P, I32, I32, PI32, PI32, PI64, PI32, PP],
    "mpsg_symmatrix": [P, P, I32, PI32, I32, PI32, PP],
    "mpsg_matmul": [P, P, P, I32, PP],
    "mpsg_contract": [P, P, PI32, P, PI32, I32, PP, PF64],
    "mpsg_contract_flops": [P, P, PI32, P, PI32, PF64],
    "mpsg_contract_noalloc": [P, P, PI32, P, PI32, P],
    "mpsg_contract_complex": [P, P, P, F64, PI32, P, P, F64, PI32, I32, PP, PP, PF64, PF64],
    "mpsg_applymps2site": [P, P, P, P, P, P, I32, PP],
    "mpsg_applymps2site_host": [P, P, P, P, P, P, P, P, P, P, P, I32, P, PP],
    "mpsg_applymps2site_flops": [P, P, P, P, P, P, PF64],
    "mpsg_mpsupdateleft": [P, P, P, P, I32, PP],
    "mpsg_mpsupdateright": [P, P, P, P, I32, PP],
    "mpsg_svd": [P, P, PP, PP, PP],
    "mpsg_svdtrunc": [P, P, I64, F64, F64, PP, PP, PP],
    "mpsg_svdtrunc_gram": [P, P, I64, F64, F64, I32, PP, PP, PP],
    "mpsg_svd_complex": [P, P, P, I32, I64, F64, F64, PP, PP, PP, PP, PP],
    "mpsg_dots": [P, I32, PP, PP, PF64],
    "mpsg_lincomb": [P, I32, PF64, PP, P],
    "mpsg_truncatedsizes": [I32, PI64, PF64, I64, F64, F64, PI64],
    "mpsg_small_eigh": [I32, PF64, PF64, PF64],
    "mpsg_eigsolve_heff2": [P, P, P, P, P, P, I32, I32, F64, I32, PF64, PP, PF64, PI32, PI32,
                            PI32],
    "mpsg_heff2_create": [P, P, P, P, P, P, I32, PP],
    "mpsg_heff2_apply": [P, P, P, PP],
    "mpsg_heff2_traffic": [P, PF64, PF64],
    "mpsg_heff2_flops": [P, PF64],
    "mpsg_heff2_free": [P],
    "mpsg_plan_heff2_check": [P, P, P, P, P],
    "mpsg_heff2_batch_create": [P, I32, PP, PP, PP, PP, PP, I32, I32, PP],
    "mpsg_heff2_batch_apply": [P, PP, PP],
    "mpsg_heff2_prepare": [P, P, P, P, P, P, I32, PP],
    "mpsg_heff2_batch_from": [P, I32, PP, I32, PP],
    "mpsg_heff2_batch_eigsolve": [P, PP, I32, I32, F64, PF64, PP, PF64, PI32, PI32, PI32],
    "mpsg_heff2_batch_info": [P, PF64, PI64, PI64, PI32],
    "mpsg_heff2_batch_free": [P],
    "mpsg_ctx_tuner": [P, I32, PI64, PI64],
    "mpsg_ctx_set_split_tuning": [P, I32, I32, I32],
    "mpsg_meta_create": [I32, I32, PI32, PI32, PI64, PI32, PP],
    "mpsg_plan_permutelegs": [P, PI32, PP],
    "mpsg_plan_fuselegs": [P, I32, I32, I32, PP],
    "mpsg_plan_splitleg": [P, I32, I32, PI32, PI32, PI64, PI32, PP],
    "mpsg_plan_symmatrix": [P, I32, PI32, I32, PI32, PP],
    "mpsg_plan_matmul": [P, P, PP, PF64],
    "mpsg_plan_contract": [P, PI32, P, PI32, PP, PF64],
    "mpsg_plan_contract_tasks": [P, PI32, P, PI32, PI64, PI64],
    "mpsg_plan_contract_gemms": [P, PI32, P, PI32, PI64, PI64],
    "mpsg_fill": [P, P, F64],
    "mpsg_rmul": [P, P, F64],
    "mpsg_mul": [P, P, P, F64],
    "mpsg_axpy": [P, F64, P, P],
    "mpsg_axpby": [P, F64, P, F64, P],
    "mpsg_dot": [P, P, P, PF64],
    "mpsg_norm": [P, P, PF64],
}


def _load():
    # MPSG_LIBRARY=checked selects the device-checked debug library (same ABI)
    checked = os.environ.get("MPSG_LIBRARY", "") == "checked"
    path = _build.build(checked=checked)  # no-op when the in-tree library is up to date
    lib = C.CDLL(path)
    for name, argt in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = argt
        fn.restype = C.c_int
    lib.mpsg_last_error.argtypes = []
    lib.mpsg_last_error.restype = C.c_char_p
    return lib, path


lib, LIB_PATH = _load()


def check(rc: int):
    if rc != OK:
        msg = lib.mpsg_last_error().decode(errors="replace")
        raise _ERRORS.get(rc, MPSGError)(rc, msg)


def call(name: str, *args):
    check(getattr(lib, name)(*args))


def i32arr(vals):
    vals = list(vals)
    return (C.c_int32 * max(1, len(vals)))(*vals)


def i64arr(vals):
    vals = list(vals)
    return (C.c_int64 * max(1, len(vals)))(*vals)
