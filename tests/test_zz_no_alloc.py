"""mpsg_contract_noalloc: the allocation-free FP64 contraction, against mpsg_contract.

Both entry points run the same planner and kernels; the no-alloc one keeps its task tables and
fused operands in a fixed device array instead of allocated buffers. The results must agree to
the FP64 contraction tolerance on consecutive calls of different shapes (the array keeps the
previous call's contents). Collected last so that it also runs after every other GPU test.
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
