"""Failure paths on the GPU without a fault: non-convergence is reported, not hidden; NaN inputs
propagate or raise, never hang; the context keeps working after every error."""
import numpy as np
import pytest

import mps_gb300 as mg
from mps_gb300 import dmrg as gd
from helpers import rand_tensor, to_device
from oracle.symtensors import U1Space, dual_space

pytestmark = pytest.mark.gpu


def test_lanczos_reports_non_convergence():
    v, eL, eR, W1, W2 = gd.heff_problem(64, 0.5, 1911, ncharges=9)
    e, x, info = mg.eigsolve_heff2(v, eL, eR, W1, W2, krylovdim=2, maxiter=1, tol=1e-15)
    assert not info.converged and np.isfinite(e) and info.normres > 1e-15
    e2, x2, info2 = mg.eigsolve_heff2(v, eL, eR, W1, W2, krylovdim=8, maxiter=60, tol=1e-10)
    assert info2.converged and e2 <= e + 1e-12


def test_nan_input_propagates_and_context_survives():
    v, eL, eR, W1, W2 = gd.heff_problem(64, 0.5, 1911, ncharges=9)
    ok = mg.applymps2site(v, eL, eR, W1, W2, precision=0).to_flat()
    bad = v.to_flat()
    bad[7] = np.nan
    vb = mg.from_flat(v.charge, v.space, bad)
    for S in (0, 3, 4, 7):  # FP64, fast and exact split modes: NaN reaches the output
        out = mg.applymps2site(vb, eL, eR, W1, W2, precision=S).to_flat()
        assert np.isnan(out).any()
        # the other outputs stay the FP64 values (to the slicing accuracy)
        fin = np.isfinite(out)
        assert fin.sum() > 0
        assert np.linalg.norm(out[fin] - ok[fin]) < 1e-4 * np.linalg.norm(ok[fin])
    again = mg.applymps2site(v, eL, eR, W1, W2, precision=0).to_flat()
    np.testing.assert_array_equal(again, ok)


@pytest.mark.parametrize("method", ["exact", "gram_left"])
def test_svd_of_a_nan_block_returns_or_raises_and_context_survives(method):
    rng = np.random.default_rng(2)
    V, W = U1Space((0, 6), (1, 5)), U1Space((0, 4), (1, 7), isdual=True)
    A = rand_tensor(0, (V, W), rng)
    good = to_device(A)
    flat = good.to_flat()
    flat[3] = np.nan
    bad = mg.from_flat(good.charge, good.space, flat)
    try:  # either a status (non-convergence) or a result: what matters is that it returns
        mg.svdtrunc(bad, maxdim=20, tol=0.0, method=method)
    except mg.MPSGError:
        pass
    u, s, v = mg.svdtrunc(good, maxdim=20, tol=0.0, method=method)
    recon = mg.matmul(mg.matmul(u, s, precision=0), v, precision=0).to_flat()
    assert np.linalg.norm(recon - good.to_flat()) < 1e-12 * np.linalg.norm(good.to_flat())
