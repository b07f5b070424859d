"""CPU checks of the library's host-side numerics: the truncation rule (src/mpsutils.jl:89-112)
against the oracle, including ties and the absolute tolerance, and the small symmetric
eigensolver used on the Lanczos projected matrix."""
import numpy as np
import pytest

import mps_gb300 as mg
from oracle import symtensors as st


@pytest.mark.parametrize("seed", range(20))
def test_truncatedsizes_matches_oracle(seed):
    rng = np.random.default_rng(seed)
    nsec = int(rng.integers(1, 8))
    S = [np.sort(rng.random(int(rng.integers(1, 12))))[::-1] for _ in range(nsec)]
    if seed % 3 == 0:  # exact ties across sectors, as SU(2) multiplets produce
        S = [s.copy() for s in S]
        for i in range(1, nsec):
            S[i][: min(len(S[i]), len(S[0]))] = S[0][: min(len(S[i]), len(S[0]))]
    maxdim = int(rng.integers(1, 30))
    tol = float(rng.choice([1e-14, 0.05, 0.3]))
    if max(s[0] for s in S) < tol:
        with pytest.raises(mg.MPSGError):
            mg.truncatedsizes(S, maxdim=maxdim, tol=tol)
        return
    for band in (0.0, 1e-12):
        assert mg.truncatedsizes(S, maxdim=maxdim, tol=tol, tieband=band) == \
            st.truncatedsizes(S, maxdim=maxdim, tol=tol, tieband=band)


def test_truncatedsizes_tieband_breaks_near_ties_by_sector_order():
    S = [np.array([1.0, 0.5 - 1e-15]), np.array([1.0, 0.5 + 1e-15])]
    assert mg.truncatedsizes(S, maxdim=3, tol=0.0) == [1, 2]          # reference rule
    assert mg.truncatedsizes(S, maxdim=3, tol=0.0, tieband=1e-12) == [2, 1]


def test_truncatedsizes_error_when_all_below_tol():
    with pytest.raises(mg.MPSGError) as e:
        mg.truncatedsizes([np.array([1e-3])], maxdim=4, tol=1e-2)
    assert e.value.code == 6


@pytest.mark.parametrize("n", [1, 2, 5, 9, 20])
def test_small_eigh_matches_numpy(n):
    rng = np.random.default_rng(n)
    A = rng.standard_normal((n, n))
    A = A + A.T
    w, v = mg.small_eigh(A)
    w0 = np.linalg.eigvalsh(A)
    np.testing.assert_allclose(w, w0, atol=1e-12 * max(1, np.abs(w0).max()))
    np.testing.assert_allclose(A @ v, v * w, atol=1e-11 * max(1, np.abs(w0).max()))
