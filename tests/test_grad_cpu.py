"""Adjoint contractions and the energy-gradient tape on the CPU oracle backend.

The tape logic (labels of the adjoint contractions, duals, accumulation) is backend independent;
here it runs on the oracle and is checked against central finite differences (exact up to
rounding for the multilinear maps involved) and, for dE/dDelta, against finite differences of
exact-diagonalisation ground energies (Hellmann-Feynman at a converged DMRG state).
"""
import numpy as np
import pytest

from mps_gb300 import grad as gr
from oracle import mps as om
from oracle import symtensors as st
from oracle.symtensors import U1Space, dual_space as dual

from helpers import rand_tensor


def oracle_backend():
    return gr.Backend(st.contract, st.dual, st.permutelegs, st.axpy, st.scaled,
                      lambda a, b: float(np.real(st.dot(a, b))))


def perturbed(T, D, h):
    return st.axpy(h, D, st.scaled(T, 1.0))


PATTERNS = [  # (ia, ib) over rank-3 A and rank-4 B: the H_eff / environment shapes
    ((-1, 2, 1), (-1, 3, 4, 5)),
    ((1, -1, -2), (-2, 2, -1, 3)),
    ((-1, -2, 1), (-2, -1, 2, 3)),
    ((2, -1, 1), (3, -1, 4, 5)),
]


@pytest.mark.parametrize("k", range(len(PATTERNS)))
def test_contract_vjp_matches_finite_differences(k):
    rng = np.random.default_rng(k)
    ia, ib = PATTERNS[k]
    V = [U1Space((0, 2), (1, 3), (2, 2)) for _ in range(7)]
    # A's and B's legs: contracted pairs are dual of each other
    la = {}
    spa = []
    for j, lab in enumerate(ia):
        sp = V[j]
        spa.append(sp)
        la[lab] = sp
    spb = [dual(la[lab]) if lab < 0 else V[3 + j] for j, lab in enumerate(ib)]
    A = rand_tensor(0, tuple(spa), rng)
    B = rand_tensor(0, tuple(spb), rng)
    Cc = st.contract(A, ia, B, ib)
    R = rand_tensor(Cc.charge, Cc.space, rng)
    be = oracle_backend()
    dA, dB = gr.contract_vjp(be, A, ia, B, ib, R)
    assert dA.space == A.space and dA.charge == A.charge
    assert dB.space == B.space and dB.charge == B.charge
    f = lambda a, b: float(st.dot(R, st.contract(a, ia, b, ib)))
    for X, dX, which in ((A, dA, 0), (B, dB, 1)):
        D = rand_tensor(X.charge, X.space, rng)
        h = 1e-3
        if which == 0:
            fd = (f(perturbed(A, D, h), B) - f(perturbed(A, D, -h), B)) / (2 * h)
        else:
            fd = (f(A, perturbed(B, D, h)) - f(A, perturbed(B, D, -h))) / (2 * h)
        assert abs(float(st.dot(dX, D)) - fd) <= 1e-10 * max(1.0, abs(fd))


def test_full_contraction_vjp():
    rng = np.random.default_rng(9)
    V1, V2 = U1Space((0, 3), (1, 2)), U1Space((-1, 2), (0, 4))
    A = rand_tensor(0, (V1, V2), rng)
    B = rand_tensor(0, (dual(V2), dual(V1)), rng)
    be = oracle_backend()
    dA, dB = gr.contract_vjp(be, A, (-1, -2), B, (-2, -1), 2.5)
    D = rand_tensor(0, A.space, rng)
    h = 1e-3
    f = lambda a: float(st.contract(a, (-1, -2), B, (-2, -1)))
    fd = (f(perturbed(A, D, h)) - f(perturbed(A, D, -h))) / (2 * h)
    assert abs(float(st.dot(dA, D)) - 2.5 * fd) < 1e-10 * max(1.0, abs(fd))


def boundaries(As, Ws):
    lVa, rVa = As[0].space[0], dual(As[-1].space[2])
    lVw, rVw = Ws[0].space[0], dual(Ws[-1].space[2])
    return (st.fill(1.0, 0, (dual(lVa), dual(lVw), lVa)),
            st.fill(1.0, 0, (rVa, rVw, dual(rVa))))


def converged_chain(lx, delta, seed=3):
    M = lx // 2
    rng = np.random.default_rng(seed)
    d = U1Space((0, 1), (1, 1))
    Vl = U1Space((0, 1))
    As = []
    for site in range(1, lx + 1):
        Vr = U1Space(*om.binomial_bond_dims(lx, site, M, 64))
        As.append(rand_tensor(0, (Vl, d, dual(Vr)), rng))
        Vl = Vr
    mps = om.MPState(As, 0)
    om.center_at(mps, 1)
    Ws = om.xxz_u1mpo(lx, delta)
    env = om.initialenv(mps, Ws)
    for _ in range(3):
        om.dmrg2sitesweep(mps, Ws, env, maxdim=64, tol=1e-13, krylovdim=6, krylovmaxiter=30,
                          lanczostol=1e-12)
    return mps, Ws


def energy_and_tape(As, Ws):
    be = oracle_backend()
    tape = gr.Tape(be)
    Lb, Rb = boundaries(As, Ws)
    E = gr.mpo_expectation(tape, As, Ws, Lb, Rb)
    return float(E), tape, E


def test_energy_gradients_site_tensor_and_delta():
    """dE/dA_l (directional, vs central differences of <psi|H|psi>) and dE/dDelta by
    Hellmann-Feynman (the tape's MPO cotangents against dW/dDelta) vs central differences of
    the exact ground energy in the Sz = 0 sector (h = 1e-5)."""
    lx, delta = 8, 0.7
    mps, Ws = converged_chain(lx, delta)
    E, tape, Eobj = energy_and_tape(mps.As, Ws)
    g = tape.backward(Eobj, 1.0)
    # ground energy by exact diagonalisation
    def e0(dl):
        H = om.xxz_hamiltonian(lx, dl)
        pop = np.array([bin(n).count("1") for n in range(2 ** lx)])
        idx = np.where(pop == lx // 2)[0]
        return np.linalg.eigvalsh(H[np.ix_(idx, idx)])[0]
    assert abs(E - e0(delta)) < 1e-9
    # site tensors: E is quadratic in A_l, so central differences are exact up to rounding
    rng = np.random.default_rng(0)
    for l in (0, 3, 7):
        A = mps.As[l]
        D = rand_tensor(A.charge, A.space, rng)
        h = 1e-4
        Ap = list(mps.As); Ap[l] = perturbed(A, D, h)
        Am = list(mps.As); Am[l] = perturbed(A, D, -h)
        fd = (energy_and_tape(Ap, Ws)[0] - energy_and_tape(Am, Ws)[0]) / (2 * h)
        assert abs(float(st.dot(g(A), D)) - fd) < 1e-8 * max(1.0, abs(fd))
    # Delta: W is linear in Delta, dW/dDelta = W(1) - W(0). The MPO may hold one tensor object
    # for several sites; the tape accumulates per object, so sum over distinct objects.
    W1, W0 = om.xxz_u1mpo(lx, 1.0), om.xxz_u1mpo(lx, 0.0)
    seen, dEd = set(), 0.0
    for W, a, b in zip(Ws, W1, W0):
        if id(W) in seen:
            continue
        seen.add(id(W))
        dEd += float(st.dot(g(W), st.axpy(-1.0, b, st.scaled(a, 1.0))))
    h = 1e-5
    fd = (e0(delta + h) - e0(delta - h)) / (2 * h)
    assert abs(dEd - fd) < 1e-6


@pytest.mark.parametrize("every", [1, 3, None, 100])
def test_checkpointed_gradients_equal_the_stored_tape(every):
    """Recomputing environments segment by segment from checkpoints gives the same energy and
    cotangents as the tape that stores every environment (site tensors and the shared MPO
    tensor objects)."""
    lx = 8
    mps, Ws = converged_chain(lx, 0.7, seed=5)
    E, tape, Eobj = energy_and_tape(mps.As, Ws)
    g = tape.backward(Eobj, 1.0)
    Lb, Rb = boundaries(mps.As, Ws)
    E2, g2 = gr.checkpointed_gradients(oracle_backend(), mps.As, Ws, Lb, Rb, every)
    assert abs(E2 - E) < 1e-13
    for X in list(mps.As) + list({id(w): w for w in Ws}.values()):
        a, b = st.flatten(g(X)), st.flatten(g2(X))
        assert np.linalg.norm(a - b) <= 1e-12 * max(1.0, np.linalg.norm(a))
