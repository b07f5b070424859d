"""Coupling derivative of a TDVP-evolved correlator on the GPU (forward-mode tangents through
the 1-site sweep on the library's complex block-sparse contractions): against central finite
differences of the GPU evolution, against the same algorithm on the CPU oracle's operations,
and against the exact derivative of exp(-iHt) at full bond dimension."""
import numpy as np
import pytest

import mps_gb300 as mg
from helpers import oracle_ops, to_device
from mps_gb300 import ctensor as ct
from mps_gb300 import dmrg as gd
from mps_gb300 import tdvp as td
from mps_gb300 import tdvp_grad as tg
from oracle import mps as om
from oracle import symtensors as st
from oracle import tdvp as ot

from test_gpu_tdvp import random_state

pytestmark = pytest.mark.gpu

DELTA, DT = 0.5, 0.05


def gpu_mpo(ops, lx, delta):
    Ws = gd.xxz_u1mpo(lx, delta)
    W1, W0 = gd.xxz_u1mpo(lx, 1.0), gd.xxz_u1mpo(lx, 0.0)
    return Ws, [ops.lincomb([(1.0, a), (-1.0, b)]) for a, b in zip(W1, W0)]


def gpu_correlator(ops, mps, lx, delta, sweeps, sites):
    Ws = gd.xxz_u1mpo(lx, delta)
    As = [ct.CTensor(to_device(A)) for A in mps.As]
    env = td.initialenv(ops, As, Ws)
    for _ in range(sweeps):
        td.tdvp1sitesweep(ops, DT, As, Ws, env, turning="symmetric")
    sz = td.site_operator(ops, mg.VectorSpace(gd.SITE), {0: -0.5, 1: 0.5})
    return td.expectation(ops, As, {i: sz for i in sites}).real


@pytest.mark.parametrize("lx,chimax", [(10, 6), (8, 1 << 20)])
def test_gpu_tangent_against_differences_oracle_and_exact(lx, chimax):
    mps = random_state(lx, lx // 2, chimax, seed=21)
    sites = (3, lx - 2)
    sweeps = 2
    ops = ct.gpu_ops()
    Ws, dWs = gpu_mpo(ops, lx, DELTA)
    As = [ct.CTensor(to_device(A)) for A in mps.As]
    sz = td.site_operator(ops, mg.VectorSpace(gd.SITE), {0: -0.5, 1: 0.5})
    c, dc = tg.evolve_with_tangent(ops, As, Ws, dWs, DT, sweeps, {i: sz for i in sites})
    h = 1e-5
    fd = (gpu_correlator(ops, mps, lx, DELTA + h, sweeps, sites) -
          gpu_correlator(ops, mps, lx, DELTA - h, sweeps, sites)) / (2 * h)
    assert abs(dc.real - fd) <= 1e-6 * abs(fd)
    # the same algorithm on the CPU oracle's operations
    cops = oracle_ops()
    cWs = om.xxz_u1mpo(lx, DELTA)
    cdWs = [cops.lincomb([(1.0, a), (-1.0, b)])
            for a, b in zip(om.xxz_u1mpo(lx, 1.0), om.xxz_u1mpo(lx, 0.0))]
    csz = td.site_operator(cops, mps.As[0].space[1], {0: -0.5, 1: 0.5})
    cc, cdc = tg.evolve_with_tangent(cops, [ct.CTensor(A) for A in mps.As], cWs, cdWs, DT,
                                     sweeps, {i: csz for i in sites})
    assert abs(c - cc) < 1e-11
    assert abs(dc - cdc) < 1e-9 * max(1.0, abs(cdc))
    if chimax > 1000:  # full bond dimension: symmetric 1-site TDVP is the exact evolution
        from scipy.linalg import expm_frechet
        t = 2 * DT * sweeps
        psi0 = ot.state_vector([st.array(A).astype(complex) for A in mps.As])
        H = om.xxz_hamiltonian(lx, DELTA)
        dH = om.xxz_hamiltonian(lx, 1.0) - om.xxz_hamiltonian(lx, 0.0)
        U, dU = expm_frechet(-1j * t * H, -1j * t * dH)
        psi, dpsi = U @ psi0, dU @ psi0
        idx = np.arange(psi.size)
        O = np.ones(psi.size)
        for i in sites:
            O = O * (((idx >> (lx - i)) & 1) - 0.5)
        assert abs(dc.real - 2.0 * np.vdot(psi, O * dpsi).real) < 1e-8
