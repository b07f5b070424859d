"""Energy gradients on the GPU: adjoint contractions through the C ABI against the oracle, and
dE/dDelta (Hellmann-Feynman through the MPO cotangents) of a DMRG-converged chain against
central differences of exact ground energies."""
import numpy as np
import pytest

import mps_gb300 as mg
from mps_gb300 import dmrg as gd
from mps_gb300 import grad as gr
from oracle import mps as om
from oracle import symtensors as st
from oracle.symtensors import U1Space, dual_space as dual

from helpers import to_device, to_oracle, rand_tensor, relerr
from test_grad_cpu import oracle_backend, PATTERNS

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("k", range(len(PATTERNS)))
def test_gpu_contract_vjp_matches_oracle(k):
    rng = np.random.default_rng(20 + k)
    ia, ib = PATTERNS[k]
    V = [U1Space((0, 20), (1, 33), (2, 17)) for _ in range(7)]
    la, spa = {}, []
    for j, lab in enumerate(ia):
        spa.append(V[j])
        la[lab] = V[j]
    spb = [dual(la[lab]) if lab < 0 else U1Space((0, 2), (1, 3)) for lab in ib]
    A = rand_tensor(0, tuple(spa), rng)
    B = rand_tensor(0, tuple(spb), rng)
    R = rand_tensor(0, st.contract(A, ia, B, ib).space, rng)
    dA0, dB0 = gr.contract_vjp(oracle_backend(), A, ia, B, ib, R)
    dA, dB = gr.contract_vjp(gr.gpu_backend(), to_device(A), ia, to_device(B), ib, to_device(R))
    assert relerr(dA.to_flat(), st.flatten(dA0)) < 1e-12
    assert relerr(dB.to_flat(), st.flatten(dB0)) < 1e-12


def test_gpu_energy_gradient_delta_and_site_tensors():
    lx, delta, chi = 12, 0.8, 64
    Ws = gd.xxz_u1mpo(lx, delta)
    mps = gd.mps_from_host(gd.random_mps_host(lx, lx // 2, chi, seed=5))
    gd.center_at(mps, 1)
    env = gd.initialenv(mps, Ws)
    for _ in range(4):
        gd.dmrg2sitesweep(mps, Ws, env, maxdim=chi, tol=1e-13, lanczostol=1e-12, krylovdim=6,
                          krylovmaxiter=30)
    E, g = gr.energy_gradients(mps.As, Ws)
    H = om.xxz_hamiltonian(lx, delta)
    pop = np.array([bin(n).count("1") for n in range(2 ** lx)])
    idx = np.where(pop == lx // 2)[0]

    def e0(dl):
        Hd = om.xxz_hamiltonian(lx, dl)
        return np.linalg.eigvalsh(Hd[np.ix_(idx, idx)])[0]

    assert abs(E - e0(delta)) < 1e-9
    dEd = gr.xxz_delta_derivative(g, Ws, lx)
    h = 1e-5
    assert abs(dEd - (e0(delta + h) - e0(delta - h)) / (2 * h)) < 1e-6
    # a converged state is stationary: dE/dA_l = 2 E A_l at the normalised center (l = 1)
    gA = g(mps.As[0])
    assert relerr(gA.to_flat(), 2 * E * mps.As[0].to_flat()) < 1e-6
    # the checkpointed backward sweep (environments recomputed per segment) gives the same
    E2, g2 = gr.energy_gradients_checkpointed(mps.As, Ws, every=4)
    assert abs(E2 - E) < 1e-12 * abs(E)
    for X in list(mps.As) + list({id(w): w for w in Ws}.values()):
        assert relerr(g2(X).to_flat(), g(X).to_flat()) < 1e-12
