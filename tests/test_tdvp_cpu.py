"""Time evolution on the CPU: the dense TDVP oracle (src/tdvp.jl restated) against exact
diagonalisation, and the library's symmetric complex TDVP host logic (``mps_gb300.tdvp`` on the
oracle's real operations) against the dense oracle."""
import numpy as np
import pytest

from helpers import dense_site, oracle_ops, rand_tensor
from mps_gb300 import ctensor as ct
from mps_gb300 import tdvp as td
from oracle import mps as om
from oracle import symtensors as st
from oracle import tdvp as ot
from oracle.symtensors import U1Space, dual_space

LX, M, DELTA, DT = 8, 4, 0.5, 0.05


def random_state(lx, m, chimax, seed):
    """Random U(1) MPS (total charge m), canonicalised to center 1 and normalised."""
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


def exact_evolution(lx, delta, psi0, t):
    H = om.xxz_hamiltonian(lx, delta)
    w, Q = np.linalg.eigh(H)
    return Q @ (np.exp(-1j * t * w) * (Q.conj().T @ psi0))


def dense_state(mps):
    return [st.array(A).astype(complex) for A in mps.As]


@pytest.mark.parametrize("kind", ["1site", "2site"])
def test_dense_oracle_tdvp_is_exact_at_full_bond_dimension(kind):
    mps = random_state(LX, M, 1 << 20, seed=3)
    As = dense_state(mps)
    Ws = [st.array(W).astype(complex) for W in om.xxz_u1mpo(LX, DELTA)]
    psi0 = ot.state_vector(As)
    env = ot.initialenv(As, Ws)
    for _ in range(3):
        if kind == "1site":
            ot.tdvp1sitesweep(DT, As, Ws, env, turning="symmetric")
        else:
            ot.tdvp2sitesweep(DT, As, Ws, env, maxdim=64, tol=1e-14, turning="symmetric")
    psi = ot.state_vector(As)
    assert np.linalg.norm(psi - exact_evolution(LX, DELTA, psi0, 6 * DT)) < 1e-10


def test_dense_oracle_reference_turning_under_evolves_the_last_site():
    """The reference's schedule evolves the turning site once by dt (src/tdvp.jl:45-48) while the
    other pieces get 2 dt: at full bond dimension it is not the exact evolution."""
    mps = random_state(LX, M, 1 << 20, seed=3)
    As = dense_state(mps)
    Ws = [st.array(W).astype(complex) for W in om.xxz_u1mpo(LX, DELTA)]
    psi0 = ot.state_vector(As)
    env = ot.initialenv(As, Ws)
    ot.tdvp1sitesweep(DT, As, Ws, env, turning="reference")
    err = np.linalg.norm(ot.state_vector(As) - exact_evolution(LX, DELTA, psi0, 2 * DT))
    assert err > 1e-3


def test_exponentiate_matches_expm_on_complex_tensors():
    ops = oracle_ops()
    rng = np.random.default_rng(0)
    V = U1Space((0, 3), (1, 4), (2, 2))
    blocks = {}
    for c, n in V.sectors:
        B = rng.standard_normal((n, n))
        blocks[(c, c)] = B + B.T
    H = st.from_blocks(0, (dual_space(V), V), blocks)  # x -> x H is Hermitian
    Hd = st.array(H)
    W = (dual_space(U1Space((0, 1))), V)
    x = ct.CTensor(rand_tensor(0, W, rng), rand_tensor(0, W, rng))
    f = lambda v: ct.ccontract(ops, v, (1, -1), H, (-1, 2))
    xd = dense_site(ops, x)[0]
    w, Q = np.linalg.eigh(Hd)
    for t in (-0.3j, 0.7j, -2.0j):
        y, info = ct.exponentiate(ops, f, t, x, krylovdim=6, tol=1e-13)
        ref = xd @ (Q @ np.diag(np.exp(t * w)) @ Q.T)
        assert info.converged
        assert np.linalg.norm(dense_site(ops, y)[0] - ref) < 1e-11 * np.linalg.norm(ref)


@pytest.mark.parametrize("kind", ["1site", "2site"])
@pytest.mark.parametrize("turning", ["reference", "symmetric"])
def test_symmetric_tdvp_host_logic_matches_dense_oracle(kind, turning):
    ops = oracle_ops()
    mps = random_state(LX, M, 1 << 20, seed=5)
    As_d = dense_state(mps)
    Ws_d = [st.array(W).astype(complex) for W in om.xxz_u1mpo(LX, DELTA)]
    env_d = ot.initialenv(As_d, Ws_d)
    Ws = om.xxz_u1mpo(LX, DELTA)
    As = [ct.CTensor(A) for A in mps.As]
    env = td.initialenv(ops, As, Ws)
    for _ in range(2):
        if kind == "1site":
            ot.tdvp1sitesweep(DT, As_d, Ws_d, env_d, turning=turning)
            td.tdvp1sitesweep(ops, DT, As, Ws, env, turning=turning)
        else:
            ot.tdvp2sitesweep(DT, As_d, Ws_d, env_d, maxdim=64, tol=1e-14, turning=turning)
            td.tdvp2sitesweep(ops, DT, As, Ws, env, maxdim=64, tol=1e-14, turning=turning)
    psi_d = ot.state_vector(As_d)
    psi = ot.state_vector([dense_site(ops, A) for A in As])
    assert np.linalg.norm(psi - psi_d) < 1e-10


def test_two_point_function_of_an_evolved_state():
    ops = oracle_ops()
    mps = random_state(LX, M, 1 << 20, seed=7)
    Ws = om.xxz_u1mpo(LX, DELTA)
    As = [ct.CTensor(A) for A in mps.As]
    env = td.initialenv(ops, As, Ws)
    td.tdvp1sitesweep(ops, DT, As, Ws, env, turning="symmetric")
    psi = ot.state_vector([dense_site(ops, A) for A in As])
    d = mps.As[0].space[1]
    sz = td.site_operator(ops, d, {0: -0.5, 1: 0.5})
    for i, j in ((1, 2), (3, 6), (2, 8)):
        val = td.expectation(ops, As, {i: sz, j: sz})
        assert abs(val.imag) < 1e-12
        assert abs(val.real - ot.szsz(psi, LX, i, j)) < 1e-11
    assert abs(td.norm2(ops, As) - 1.0) < 1e-11


def _hermitian_problem(seed=0):
    ops = oracle_ops()
    rng = np.random.default_rng(seed)
    V = U1Space((0, 5), (1, 6), (2, 4))
    blocks = {}
    for c, n in V.sectors:
        B = rng.standard_normal((n, n))
        blocks[(c, c)] = B + B.T
    H = st.from_blocks(0, (dual_space(V), V), blocks)
    W = (dual_space(U1Space((0, 1))), V)
    x = ct.CTensor(rand_tensor(0, W, rng), rand_tensor(0, W, rng))
    f = lambda v: ct.ccontract(ops, v, (1, -1), H, (-1, 2))
    return ops, f, x, st.array(H)


def test_exponentiate_takes_several_steps_when_the_basis_is_small():
    """x lives in a 5-dimensional sector; a Krylov dimension of 4 cannot take t = -0.1i within
    1e-10 in one step: the step is cut, the integration restarts from the new vector, and the
    result still equals expm (a basis of 5 would be exact in one step)."""
    ops, f, x, Hd = _hermitian_problem()
    w, Q = np.linalg.eigh(Hd)
    t = -0.1j
    y, info = ct.exponentiate(ops, f, t, x, krylovdim=4, tol=1e-10, maxiter=2000)
    ref = dense_site(ops, x)[0] @ (Q @ np.diag(np.exp(t * w)) @ Q.T)
    assert info.converged and info.numsteps > 1 and info.numops == 4 * info.numsteps
    assert np.linalg.norm(dense_site(ops, y)[0] - ref) < 1e-10 * np.linalg.norm(ref)
    y5, info5 = ct.exponentiate(ops, f, t, x, krylovdim=5, tol=1e-10)
    assert info5.numsteps == 1
    assert np.linalg.norm(dense_site(ops, y5)[0] - ref) < 1e-12 * np.linalg.norm(ref)


def test_exponentiate_reports_an_unfinished_integration():
    ops, f, x, _ = _hermitian_problem()
    y, info = ct.exponentiate(ops, f, -3.0j, x, krylovdim=2, tol=1e-14, maxiter=1)
    assert not info.converged and info.numsteps == 1


def test_exponentiate_of_zero_is_zero():
    ops, f, x, _ = _hermitian_problem()
    z = ct.cscale(ops, x, 0.0)
    y, info = ct.exponentiate(ops, f, -1.0j, z)
    assert info.converged and info.numops == 0
    assert np.all(dense_site(ops, y)[0] == 0)
