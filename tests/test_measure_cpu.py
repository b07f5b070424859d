"""Measurements (src/symmps.jl:202-221,245-371,452-482) on the oracle's operations against
dense state vectors: local and two-point functions, MPO expectation, overlap, norm, Schmidt
values; for a real MPS and for a complex (time-evolved) one."""
import numpy as np
import pytest

from helpers import dense_site, oracle_ops, rand_tensor
from mps_gb300 import ctensor as ct
from mps_gb300 import measure as ms
from mps_gb300 import tdvp as td
from oracle import mps as om
from oracle import symtensors as st
from oracle import tdvp as ot
from oracle.symtensors import U1Space, dual_space

LX, M = 8, 4


def random_mps(lx, m, chimax, seed, canonical=True):
    rng = np.random.default_rng(seed)
    d = U1Space((0, 1), (1, 1))
    Vl = U1Space((0, 1))
    As = []
    for site in range(1, lx + 1):
        Vr = U1Space(*om.binomial_bond_dims(lx, site, m, chimax))
        As.append(rand_tensor(0, (Vl, d, dual_space(Vr)), rng))
        Vl = Vr
    mps = om.MPState(As, 0)
    if canonical:
        om.center_at(mps, 1)
        mps.As[0] = st.scaled(mps.As[0], 1.0 / st.norm(mps.As[0]))
    return mps


def sz_diag(lx, i):
    idx = np.arange(2 ** lx)
    return ((idx >> (lx - i)) & 1) - 0.5


def states(ops):
    """(site list, dense state vector) for a real canonical MPS and a complex evolved one."""
    mps = random_mps(LX, M, 6, seed=21)
    real = list(mps.As)
    psi_r = ot.state_vector([st.array(A) for A in real])
    Ws = om.xxz_u1mpo(LX, 0.7)
    As = [ct.CTensor(A) for A in random_mps(LX, M, 6, seed=22).As]
    env = td.initialenv(ops, As, Ws)
    td.tdvp1sitesweep(ops, 0.1, As, Ws, env, turning="symmetric")
    psi_c = ot.state_vector([dense_site(ops, A) for A in As])
    return [(real, psi_r), (As, psi_c)]


@pytest.mark.parametrize("which", [0, 1])
def test_local_and_two_point_functions(which):
    ops = oracle_ops()
    As, psi = states(ops)[which]
    sz = td.site_operator(ops, U1Space((0, 1), (1, 1)), {0: -0.5, 1: 0.5})
    p = np.abs(psi) ** 2
    loc = ms.measure_site(As, sz, ops=ops)
    for x in range(1, LX + 1):
        assert abs(loc[x] - np.sum(p * sz_diag(LX, x))) < 1e-12
    assert ms.measure_site(As, sz, 3, ops=ops)[3] == pytest.approx(loc[3], abs=1e-14)
    pairs = ms.measure_pairs(As, sz, sz, ops=ops)
    assert len(pairs) == LX * (LX - 1) // 2
    for (a, b), v in pairs.items():
        assert abs(v - np.sum(p * sz_diag(LX, a) * sz_diag(LX, b))) < 1e-12
    one = ms.measure_pairs(As, sz, sz, 2, 7, ops=ops)
    assert one[(2, 7)] == pytest.approx(pairs[(2, 7)], abs=1e-14)


@pytest.mark.parametrize("which", [0, 1])
def test_mpo_expectation_overlap_and_norm(which):
    ops = oracle_ops()
    As, psi = states(ops)[which]
    H = om.xxz_hamiltonian(LX, 0.3)
    e = ms.measure_mpo(As, om.xxz_u1mpo(LX, 0.3), ops=ops)[1]
    assert abs(e - np.vdot(psi, H @ psi)) < 1e-11
    assert ms.norm(As, ops=ops) == pytest.approx(np.linalg.norm(psi), rel=1e-13)
    other, phi = states(ops)[1 - which]
    assert abs(ms.overlap(As, other, ops=ops) - np.vdot(phi, psi)) < 1e-12


def test_schmidt_values_and_entropy():
    ops = oracle_ops()
    As, psi = states(ops)[0]
    sv = ms.schmidtvalues(As, ops=ops)
    ent = ms.entanglemententropy(As, ops=ops)
    for l in range(1, LX):
        s = np.linalg.svd(psi.reshape(2 ** l, 2 ** (LX - l)), compute_uv=False)
        s = s[s > 1e-13 * s[0]]
        got = np.asarray(sv[l - 1])
        got = got[got > 1e-13 * got[0]]
        np.testing.assert_allclose(got, s, rtol=1e-10, atol=1e-13)
        pr = s ** 2
        assert ent[l - 1] == pytest.approx(-np.sum(pr * np.log(pr)), abs=1e-10)


def test_charged_two_point_function():
    """<S+_i S-_j> (operator charges +1 and -1, src/symmps.jl:312-343 allows charges summing to
    zero) against the dense state vector, for a real and a complex state."""
    ops = oracle_ops()
    d = U1Space((0, 1), (1, 1))
    sp = td.site_operator(ops, d, np.array([[0.0, 0.0], [1.0, 0.0]]), charge=1)
    sm = td.site_operator(ops, d, np.array([[0.0, 1.0], [0.0, 0.0]]), charge=-1)
    for As, psi in states(ops):
        got = ms.measure_pairs(As, sp, sm, ops=ops)
        idx = np.arange(2 ** LX)
        for (i, j), v in got.items():
            bi, bj = 1 << (LX - i), 1 << (LX - j)
            # S-_j then S+_i: j up -> down, then i down -> up
            src = idx[((idx & bj) != 0) & ((idx & bi) == 0)]
            dst = src - bj + bi
            want = np.vdot(psi[dst], psi[src])
            assert abs(v - want) < 1e-12, (i, j)
