"""The benchmark workload itself against the oracle: one two-site H_eff application
(src/apply.jl:93-105) at chi = 2048 on both bonds (25 charges, binomial profile, XXZ Delta = 0.5,
Philox seed 1911), through every path the library offers for it.

The oracle (NumPy/OpenBLAS restatement of the reference's four contractions) builds its inputs
from its own Philox draws (``oracle.mps.heff_workload``); the device tensors come from the
library's generator, and the first test checks that both are the same numbers.  Tolerances:
FP64 paths 1e-12 relative (Frobenius over the whole result); split precision S slices the
4x slicing bound used by the small-size split tests.
"""
import numpy as np
import pytest
import torch

import mps_gb300 as mg
from mps_gb300 import dmrg as gd
from oracle import mps as om
from oracle import symtensors as st

from helpers import relerr

pytestmark = pytest.mark.gpu

CHI = 2048
RTOL64 = 1e-12
# slicing bounds of the split-precision products (as in test_gpu_split.py, exact mode)
TOL = {4: 2e-8, 5: 2e-10, 6: 2e-12, 7: 1e-13}


@pytest.fixture(scope="module")
def workload():
    O = list(om.heff_workload(CHI))
    want = st.flatten(om.applymps2site(*O))
    D = list(gd.heff_problem(CHI))
    return O, D, want


def test_inputs_are_the_oracles(workload):
    O, D, _ = workload
    for T, Dt in zip(O, D):
        assert Dt.sectors() == T.sectors()
        assert np.array_equal(Dt.to_flat(), st.flatten(T))


def test_flops_equal_the_oracles_count(workload):
    O, D, _ = workload
    assert mg.applymps2site_flops(*D) == om.heff_flops(*O)


def test_fp64_drop_in_full_size(workload):
    _, D, want = workload
    got = mg.applymps2site(*D, precision=0).to_flat()
    assert relerr(got, want) <= RTOL64, relerr(got, want)


def test_fp64_prepared_operator_full_size(workload):
    _, D, want = workload
    op = mg.Heff2(*D, precision=0)
    for _ in range(2):  # a second application reuses the prepared plans
        got = op(D[0]).to_flat()
        assert relerr(got, want) <= RTOL64, relerr(got, want)


@pytest.mark.parametrize("S", [4, 7])
def test_split_operator_full_size(workload, S):
    _, D, want = workload
    op = mg.Heff2(*D, precision=S)
    e = relerr(op(D[0]).to_flat(), want)
    assert e < 4 * TOL[S], e


@pytest.mark.parametrize("S", [0, 4])
def test_host_buffer_call_full_size(workload, S):
    O, _, want = workload
    ctx = mg.get_context()
    dev = [mg.zeros(T.charge, tuple(mg.VectorSpace(V.sectors, V.isdual) for V in T.space), ctx)
           for T in O]
    host_in = [torch.from_numpy(st.flatten(T).copy()).pin_memory() for T in O]
    host_out = torch.full((dev[0].numel(),), float("nan"), dtype=torch.float64).pin_memory()
    for _ in range(2):
        host_out.fill_(float("nan"))
        mg.applymps2site_host(*dev, host_in, host_out, precision=S)
        e = relerr(host_out.numpy(), want)
        assert e <= (RTOL64 if S == 0 else 4 * TOL[S]), e
