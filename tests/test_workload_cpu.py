"""The benchmark's H_eff input as the oracle states it and as the library generates it: the same
bond profile, the same Philox draws in the same block order, and the same algorithmic flop count
(the oracle counts its own sector GEMMs; the library's planner counts its GEMM tasks).  The
reference arm of bench.py relies on this to time the oracle without loading the library."""
import numpy as np
import pytest

from mps_gb300 import dmrg as gd
from oracle import mps as om
from oracle import symtensors as st


@pytest.mark.parametrize("chi,nq", [(16, 5), (64, 9), (256, 13), (1000, 8), (2048, 25),
                                    (4096, 25)])
def test_profile(chi, nq):
    p = om.binomial_profile(chi, nq)
    assert p == gd.binomial_profile(chi, nq)
    assert sum(p) == chi and min(p) >= 1 and p == p[::-1]


@pytest.mark.parametrize("chi,nq", [(64, 9), (2048, 25)])
def test_inputs_and_flops(chi, nq):
    O = om.heff_workload(chi, 0.5, 1911, nq)
    (sv, sl, sr), flats = gd.heff_inputs_host(chi, 0.5, 1911, nq)
    for T, sp, f in zip(O[:3], (sv, sl, sr), flats):
        assert tuple(st.VectorSpace(V.sectors, V.isdual) for V in sp) == T.space
        assert np.array_equal(st.flatten(T), f)
    meta = gd.heff_problem(chi, meta_only=True, ncharges=nq)
    assert om.heff_flops(*O) == gd.heff_flops_meta(*meta)


def test_full_size_flop_count():
    """9.4736 GFLOP per application at chi = 2048 (the figure every GFLOP/s number uses)."""
    assert om.heff_flops(*om.heff_workload(2048)) == 9473552944.0


def test_flop_counter_counts_only_present_pairs():
    V = st.U1Space((0, 3), (1, 2))
    A = st.fill(1.0, 0, (V, st.dual_space(V)))
    B = st.fill(1.0, 0, (V, st.dual_space(V)))
    with st.FlopCount() as fc:
        st.matmul(A, B)
    assert fc.flops == 2 * 3 * 3 * 3 + 2 * 2 * 2 * 2
    with st.FlopCount() as outer:
        with st.FlopCount() as inner:
            st.matmul(A, B)
        st.matmul(A, B)
    assert inner.flops == fc.flops and outer.flops == 2 * fc.flops
