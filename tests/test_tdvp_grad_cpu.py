"""Coupling derivatives of TDVP-evolved correlators (forward-mode tangents through the 1-site
sweep, ``mps_gb300.tdvp_grad``) on the CPU, with the oracle's real operations: against central
finite differences (h = 1e-5) of the same evolution on a truncated chain, and against the exact
derivative of exp(-iHt) (Frechet derivative of the dense matrix exponential) where 1-site TDVP
with the symmetric turning point is the exact evolution (full bond dimension)."""
import numpy as np
import pytest

from helpers import dense_site, oracle_ops, rand_tensor
from mps_gb300 import ctensor as ct
from mps_gb300 import tdvp as td
from mps_gb300 import tdvp_grad as tg
from oracle import mps as om
from oracle import symtensors as st
from oracle import tdvp as ot
from oracle.symtensors import U1Space, dual_space

LX, M, DELTA, DT = 8, 4, 0.5, 0.05


def random_state(lx, m, chimax, seed):
    rng = np.random.default_rng(seed)
    d = U1Space((0, 1), (1, 1))
    Vl = U1Space((0, 1))
    As = []
    for site in range(1, lx + 1):
        Vr = U1Space(*om.binomial_bond_dims(lx, site, m, chimax))
        As.append(rand_tensor(0, (Vl, d, dual_space(Vr)), rng))
        Vl = Vr
    mps = om.center_at(om.MPState(As, 0), 1)
    mps.As[0] = st.scaled(mps.As[0], 1.0 / st.norm(mps.As[0]))
    return mps


def mpo_and_derivative(ops, lx, delta):
    Ws = om.xxz_u1mpo(lx, delta)
    W1, W0 = om.xxz_u1mpo(lx, 1.0), om.xxz_u1mpo(lx, 0.0)
    return Ws, [ops.lincomb([(1.0, a), (-1.0, b)]) for a, b in zip(W1, W0)]


def correlator(ops, mps, delta, sweeps, sites, turning="symmetric"):
    Ws = om.xxz_u1mpo(LX, delta)
    As = [ct.CTensor(A) for A in mps.As]
    env = td.initialenv(ops, As, Ws)
    for _ in range(sweeps):
        td.tdvp1sitesweep(ops, DT, As, Ws, env, turning=turning)
    sz = td.site_operator(ops, mps.As[0].space[1], {0: -0.5, 1: 0.5})
    return td.expectation(ops, As, {i: sz for i in sites}).real, As


@pytest.mark.parametrize("turning", ["symmetric", "reference"])
def test_tangent_matches_central_differences_on_a_truncated_chain(turning):
    ops = oracle_ops()
    mps = random_state(LX, M, 4, seed=11)
    sites = (3, 6)
    Ws, dWs = mpo_and_derivative(ops, LX, DELTA)
    As = [ct.CTensor(A) for A in mps.As]
    sz = td.site_operator(ops, mps.As[0].space[1], {0: -0.5, 1: 0.5})
    c, dc = tg.evolve_with_tangent(ops, As, Ws, dWs, DT, 2, {i: sz for i in sites},
                                   turning=turning)
    c0, As0 = correlator(ops, mps, DELTA, 2, sites, turning)
    # the state carried by the tangent sweep is the plain sweep's
    for A, B in zip(As, As0):
        assert np.abs(dense_site(ops, A) - dense_site(ops, B)).max() < 1e-12
    assert abs(c.real - c0) < 1e-12
    h = 1e-5
    fd = (correlator(ops, mps, DELTA + h, 2, sites, turning)[0] -
          correlator(ops, mps, DELTA - h, 2, sites, turning)[0]) / (2 * h)
    assert abs(dc.real - fd) <= 1e-6 * abs(fd)
    assert abs(dc.imag) < 1e-12


def test_tangent_equals_the_exact_derivative_at_full_bond_dimension():
    ops = oracle_ops()
    from scipy.linalg import expm_frechet
    mps = random_state(LX, M, 1 << 20, seed=5)
    sites = (2, 5)
    sweeps = 3
    Ws, dWs = mpo_and_derivative(ops, LX, DELTA)
    As = [ct.CTensor(A) for A in mps.As]
    psi0 = ot.state_vector([dense_site(ops, A) for A in As])
    sz = td.site_operator(ops, mps.As[0].space[1], {0: -0.5, 1: 0.5})
    c, dc = tg.evolve_with_tangent(ops, As, Ws, dWs, DT, sweeps, {i: sz for i in sites})
    t = 2 * DT * sweeps  # a symmetric sweep is the exact evolution by 2 dt
    H = om.xxz_hamiltonian(LX, DELTA)
    dH = om.xxz_hamiltonian(LX, 1.0) - om.xxz_hamiltonian(LX, 0.0)
    U, dU = expm_frechet(-1j * t * H, -1j * t * dH)
    psi, dpsi = U @ psi0, dU @ psi0
    O = np.ones(psi.size)
    idx = np.arange(psi.size)
    for i in sites:  # Sz_i diagonal in the computational basis (site i = bit LX - i)
        O = O * (((idx >> (LX - i)) & 1) - 0.5)
    want_c = np.vdot(psi, O * psi).real
    want_dc = 2.0 * np.vdot(psi, O * dpsi).real
    assert abs(c.real - want_c) < 1e-10
    assert abs(dc.real - want_dc) < 1e-8 * max(1.0, abs(want_dc))


def test_tangent_of_the_exponential_on_its_own():
    """d/dp exp(t (F + p G)) x at p = 0 against the Frechet derivative of the dense matrix."""
    from scipy.linalg import expm_frechet
    ops = oracle_ops()
    rng = np.random.default_rng(4)
    V = U1Space((0, 5), (1, 6), (2, 4))
    fb, gb = {}, {}
    for c, n in V.sectors:
        a, b = rng.standard_normal((n, n)), rng.standard_normal((n, n))
        fb[(c, c)], gb[(c, c)] = a + a.T, b + b.T
    F = st.from_blocks(0, (dual_space(V), V), fb)
    G = st.from_blocks(0, (dual_space(V), V), gb)
    W = (dual_space(U1Space((0, 1))), V)
    x = ct.CTensor(rand_tensor(0, W, rng), rand_tensor(0, W, rng))
    f = lambda v: ct.ccontract(ops, v, (1, -1), F, (-1, 2))
    g = lambda v: ct.ccontract(ops, v, (1, -1), G, (-1, 2))
    t = -0.3j
    dy, nops, ok = tg.exponentiate_tangent(ops, f, g, t, x, None, krylovdim=8, tol=1e-12)
    assert ok
    Fd, Gd = st.array(F), st.array(G)
    xd = dense_site(ops, x)[0]
    _, L = expm_frechet(t * Fd, t * Gd)
    want = xd @ L  # row vector times the (right-acting) operator
    assert np.linalg.norm(dense_site(ops, dy)[0] - want) < 1e-11 * np.linalg.norm(want)


@pytest.mark.parametrize("turning,sweeps", [("symmetric", 2), ("reference", 1)])
def test_adjoint_matches_the_tangent_and_differences_in_the_state(turning, sweeps):
    """Reverse mode (``evolve_with_adjoint``, 6 quadrature nodes) over the sweeps of a
    truncated chain: the MPO
    cotangents contracted with dW/dDelta give the forward-mode derivative, every site's gradient
    is its own (the chain's MPO shares one tensor between its middle sites), and the cotangent
    of the initial state matches central differences along a random complex direction."""
    from mps_gb300.ctensor import cdots, clincomb
    ops = oracle_ops()
    mps = random_state(LX, M, 4, seed=11)
    sites = (3, 6)
    Ws, dWs = mpo_and_derivative(ops, LX, DELTA)
    assert len({id(W) for W in Ws}) < LX
    sz = td.site_operator(ops, mps.As[0].space[1], {0: -0.5, 1: 0.5})
    obs = {i: sz for i in sites}
    As = [ct.CTensor(A) for A in mps.As]
    c_t, dc = tg.evolve_with_tangent(ops, As, Ws, dWs, DT, sweeps, obs, turning=turning)
    As = [ct.CTensor(A) for A in mps.As]
    C, gW, gA = tg.evolve_with_adjoint(ops, As, Ws, DT, sweeps, obs, turning=turning, quad=6)
    assert abs(C - c_t) < 1e-13
    rev = sum(ops.dot(g.re, dW) for g, dW in zip(gW, dWs))
    assert abs(rev - dc.real) <= 1e-9 * abs(dc.real)
    # one site's MPO tensor alone: central differences of that site's coupling
    l, h = 4, 1e-5
    def c_site(eps):
        Wx = list(Ws)
        Wx[l - 1] = ops.lincomb([(1.0, Ws[l - 1]), (eps, dWs[l - 1])])
        As = [ct.CTensor(A) for A in mps.As]
        env = td.initialenv(ops, As, Wx)
        for _ in range(sweeps):
            td.tdvp1sitesweep(ops, DT, As, Wx, env, turning=turning)
        return td.expectation(ops, As, obs).real
    fd = (c_site(h) - c_site(-h)) / (2 * h)
    assert abs(ops.dot(gW[l - 1].re, dWs[l - 1]) - fd) <= 1e-6 * abs(fd) + 1e-10
    # the initial state
    rng = np.random.default_rng(1)
    A0 = [ct.CTensor(A) for A in mps.As]
    D = [ct.CTensor(rand_tensor(0, A.space, rng), rand_tensor(0, A.space, rng)) for A in mps.As]
    def c_state(eps):
        As = [clincomb(ops, [(1.0, a), (eps, d)]) for a, d in zip(A0, D)]
        env = td.initialenv(ops, As, Ws)
        for _ in range(sweeps):
            td.tdvp1sitesweep(ops, DT, As, Ws, env, turning=turning)
        return td.expectation(ops, As, obs).real
    fd = (c_state(h) - c_state(-h)) / (2 * h)
    an = sum(cdots(ops, [g], d)[0].real for g, d in zip(gA, D))
    assert abs(an - fd) <= 1e-6 * abs(fd) + 1e-10


@pytest.mark.parametrize("t,krylovdim", [(-0.3j, 30), (-2.0j, 8), (0.7j, 6)])
def test_exponential_family_equals_single_exponentials(t, krylovdim):
    """exp(p t F) x for several p from one integration (with restarts where the basis is short)
    against one ``exponentiate`` per p."""
    ops = oracle_ops()
    rng = np.random.default_rng(4)
    V = U1Space((0, 15), (1, 16), (2, 14))
    fb = {}
    for c, n in V.sectors:
        a = rng.standard_normal((n, n))
        fb[(c, c)] = 0.1 * (a + a.T)
    F = st.from_blocks(0, (dual_space(V), V), fb)
    W = (dual_space(U1Space((0, 1))), V)
    x = ct.CTensor(rand_tensor(0, W, rng), rand_tensor(0, W, rng))
    f = lambda v: ct.ccontract(ops, v, (1, -1), F, (-1, 2))
    fr = [0.0, 0.1, 0.35, 0.5, 0.9, 1.0]
    ys, info = tg.exponentiate_family(ops, f, t, x, fr, krylovdim=krylovdim, tol=1e-12)
    assert info.converged
    steps = 0
    for p, y in zip(fr, ys):
        if p == 0.0:
            want = x
        else:
            want, one = ct.exponentiate(ops, f, p * t, x, krylovdim=krylovdim, tol=1e-12)
            steps = max(steps, one.numsteps)
        assert np.abs(dense_site(ops, y) - dense_site(ops, want)).max() < 1e-12
    assert info.numsteps == steps  # the family costs the longest single integration
