"""mpsg_contract_noalloc: the allocation-free FP64 contraction, against mpsg_contract.

Both entry points run the same planner and kernels; the no-alloc one keeps its task tables and
fused operands in a fixed device array instead of allocated buffers. The results must agree to
the FP64 contraction tolerance on consecutive calls of different shapes (the array keeps the
previous call's contents), and a call must leave the device's memory use where it found it: the
bytes in use in the default memory pool (where stream-ordered allocations come from) and the
device's free memory (which any cudaMalloc would lower) are read through the CUDA driver before
and after. Collected last so that it also runs after every other GPU test.
"""
import ctypes as C

import numpy as np
import pytest

import mps_gb300 as mg
from mps_gb300 import _lib, dmrg as gd

from helpers import relerr

pytestmark = pytest.mark.gpu

RTOL = 1e-12

# the four contractions of the H_eff matvec (apply.jl:17-25)
STEPS = [((-1, 2, 1), (-1, 3, 4, 5)), ((1, -1, -2, 4, 5), (-1, 2, 3, -2)),
         ((1, 2, -1, -2, 5), (-1, 3, 4, -2)), ((1, 2, 3, -1, -2), (-2, -1, 4))]


def noalloc(A, ia, B, ib, out):
    _lib.call("mpsg_contract_noalloc", A.ctx.handle, A.handle, _lib.i32arr(ia), B.handle,
              _lib.i32arr(ib), out.handle)
    return out


_CU_MEMPOOL_ATTR_USED_MEM_CURRENT = 7  # CUmemPool_attribute (cuda.h)


def device_memory_in_use(device=0):
    """(bytes in use in the device's default memory pool, free bytes on the device), read with
    the driver API after the device has finished all work."""
    cu = C.CDLL("libcuda.so.1")
    assert cu.cuCtxSynchronize() == 0
    pool = C.c_void_p()
    assert cu.cuDeviceGetDefaultMemPool(C.byref(pool), C.c_int(device)) == 0
    used = C.c_uint64()
    assert cu.cuMemPoolGetAttribute(pool, C.c_int(_CU_MEMPOOL_ATTR_USED_MEM_CURRENT),
                                    C.byref(used)) == 0
    free, total = C.c_size_t(), C.c_size_t()
    assert cu.cuMemGetInfo_v2(C.byref(free), C.byref(total)) == 0
    return used.value, free.value


def heff_chain(ctx, chi, seed):
    v, eL, eR, W1, W2 = gd.heff_problem(chi, 0.5, seed, ctx, ncharges=9)
    a = [eL, None, None, None]
    b = [v, W1, W2, eR]
    return a, b


def test_noalloc_matches_contract_on_consecutive_calls():
    ctx = mg.Context(0)
    a64, b64 = heff_chain(ctx, 64, 5)
    a128, b128 = heff_chain(ctx, 128, 6)
    for a, b in ((a64, b64), (a128, b128), (a64, b64)):
        prev_ref = prev_out = None
        for k, (ia, ib) in enumerate(STEPS):
            A = a[k] if k == 0 else prev_ref
            ref = mg.contract(A, ia, b[k], ib, precision=0)
            out = mg.zeros(ref.charge, ref.space, ctx)
            mg.fill_(out, np.nan)  # every element must be written by the call
            noalloc(A, ia, b[k], ib, out)
            got, want = out.to_flat(), ref.to_flat()
            assert np.all(np.isfinite(got))
            assert relerr(got, want) <= RTOL, (k, relerr(got, want))
            # a second call in a row into a fresh output gives the same values
            out2 = noalloc(A, ia, b[k], ib, mg.zeros(ref.charge, ref.space, ctx))
            assert relerr(out2.to_flat(), want) <= RTOL
            prev_ref, prev_out = ref, out
        assert prev_out is not None


def test_noalloc_allocates_nothing():
    """Two calls in a row, after one untimed call that looks up the scratch array (and loads the
    kernels): neither changes the pool's bytes in use nor the device's free memory."""
    ctx = mg.Context(0)
    a, b = heff_chain(ctx, 128, 8)
    ia, ib = STEPS[0]
    ref = mg.contract(a[0], ia, b[0], ib, precision=0)
    outs = [mg.zeros(ref.charge, ref.space, ctx) for _ in range(3)]
    noalloc(a[0], ia, b[0], ib, outs[0])
    before = device_memory_in_use()
    noalloc(a[0], ia, b[0], ib, outs[1])
    noalloc(a[0], ia, b[0], ib, outs[2])
    after = device_memory_in_use()
    assert after == before, (before, after)
    for out in outs:
        assert relerr(out.to_flat(), ref.to_flat()) <= RTOL


def test_noalloc_rejects_what_it_cannot_do():
    ctx = mg.Context(0)
    a, b = heff_chain(ctx, 64, 7)
    ref = mg.contract(a[0], STEPS[0][0], b[0], STEPS[0][1], precision=0)
    wrong = mg.zeros(ref.charge + 2, ref.space, ctx)
    with pytest.raises(mg.MPSGError) as e:
        noalloc(a[0], STEPS[0][0], b[0], STEPS[0][1], wrong)
    assert e.value.code == _lib.ERR_SPACE_MISMATCH
    # a scalar result has no output tensor
    v = b[0]
    with pytest.raises(mg.MPSGError) as e:
        noalloc(v, (-1, -2, -3, -4), mg.dual(v), (-1, -2, -3, -4), ref)
    assert e.value.code == _lib.ERR_UNSUPPORTED
    # more than the fixed 64 MiB of scratch: a 3000 x 3000 transpose needs 72 MB fused
    V = mg.VectorSpace([(0, 3000)], False)
    big = mg.fill(1.0, 0, (V, mg.dual(V)), ctx)
    W = mg.VectorSpace([(0, 1)], False)
    vec = mg.fill(1.0, 0, (mg.dual(V), W), ctx)
    res = mg.zeros(0, (mg.dual(V), W), ctx)
    with pytest.raises(mg.MPSGError) as e:
        noalloc(big, (-1, 1), vec, (-1, 2), res)
    assert e.value.code == _lib.ERR_UNSUPPORTED
    assert "64 MiB" in str(e.value)
    # every tensor must belong to the calling context
    other = mg.Context(0)
    out_other = mg.zeros(ref.charge, ref.space, other)
    with pytest.raises(mg.MPSGError) as e:
        noalloc(a[0], STEPS[0][0], b[0], STEPS[0][1], out_other)
    assert e.value.code == _lib.ERR_ARGUMENT
    with pytest.raises(mg.MPSGError) as e:  # operands of ctx called through another context
        _lib.call("mpsg_contract_noalloc", other.handle, a[0].handle, _lib.i32arr(STEPS[0][0]),
                  b[0].handle, _lib.i32arr(STEPS[0][1]), out_other.handle)
    assert e.value.code == _lib.ERR_ARGUMENT
