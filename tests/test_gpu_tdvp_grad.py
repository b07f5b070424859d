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


def test_gpu_adjoint_against_tangent_oracle_and_differences():
    """Reverse mode on the GPU's operations (1 sweep, truncated chain): the MPO cotangents
    contracted with dW/dDelta give the forward-mode derivative; the initial state's cotangents
    equal, site by site, those of the same reverse sweep on the CPU oracle's operations (C is a
    function of the initial state whatever gauge each SVD picks, so its gradient is unique); and
    along the center site they match central differences of the GPU evolution. (Directions that
    leave the middle sites off their canonical form curve strongly: there h = 1e-5 differences
    are off by 1e-3 and only converge to the gradient for h near 1e-7.)"""
    from helpers import dense_site, rand_tensor
    lx, sweeps = 10, 1
    mps = random_state(lx, lx // 2, 6, seed=21)
    sites = (3, lx - 2)
    ops = ct.gpu_ops()
    Ws, dWs = gpu_mpo(ops, lx, DELTA)
    sz = td.site_operator(ops, mg.VectorSpace(gd.SITE), {0: -0.5, 1: 0.5})
    obs = {i: sz for i in sites}
    As = [ct.CTensor(to_device(A)) for A in mps.As]
    c, dc = tg.evolve_with_tangent(ops, As, Ws, dWs, DT, sweeps, obs)
    As = [ct.CTensor(to_device(A)) for A in mps.As]
    C, gW, gA = tg.evolve_with_adjoint(ops, As, Ws, DT, sweeps, obs, quad=6)
    assert abs(C - c) < 1e-12
    rev = sum(ops.dot(g.re, dW) for g, dW in zip(gW, dWs))
    assert abs(rev - dc.real) <= 1e-9 * abs(dc.real)
    # the same reverse sweep on the oracle
    cops = oracle_ops()
    csz = td.site_operator(cops, mps.As[0].space[1], {0: -0.5, 1: 0.5})
    cC, _, cgA = tg.evolve_with_adjoint(cops, [ct.CTensor(A) for A in mps.As],
                                        om.xxz_u1mpo(lx, DELTA), DT, sweeps,
                                        {i: csz for i in sites}, quad=6)
    assert abs(C - cC) < 1e-11
    for g, cg in zip(gA, cgA):
        a, b = dense_site(ops, g), dense_site(cops, cg)
        assert np.abs(a - b).max() <= 1e-9 * max(1.0, np.abs(b).max())
    # central differences along a random complex direction of the center site
    rng = np.random.default_rng(3)
    A1 = mps.As[0]
    dr, di = rand_tensor(0, A1.space, rng), rand_tensor(0, A1.space, rng)

    def c_center(eps):
        As = [ct.CTensor(to_device(st.axpy(eps, dr, st.scaled(A1, 1.0))),
                         to_device(st.scaled(di, eps)))]
        As += [ct.CTensor(to_device(A)) for A in mps.As[1:]]
        env = td.initialenv(ops, As, Ws)
        for _ in range(sweeps):
            td.tdvp1sitesweep(ops, DT, As, Ws, env, turning="symmetric")
        return td.expectation(ops, As, obs).real
    h = 1e-5
    fd = (c_center(h) - c_center(-h)) / (2 * h)
    an = ct.cdots(ops, [gA[0]], ct.CTensor(to_device(dr), to_device(di)))[0].real
    assert abs(an - fd) <= 1e-6 * abs(fd) + 1e-10
