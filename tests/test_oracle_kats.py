"""Pin the oracle against the reference's own known-answer tests.

Each test restates one ``@testset`` of the reference (test/symtensortests.jl, test/mpotests.jl)
with the same inputs and the same exact / approximate comparisons.  Random inputs that the
reference draws from Julia's MersenneTwister are drawn here from a seeded NumPy generator: the
tests compare against dense restatements, not against the Julia random stream.
"""
import itertools

import numpy as np
import pytest

from oracle import symtensors as st
from oracle import mps as om
from oracle.symtensors import U1Space, dual_space as dual


def rand_tensor(charge, space, rng, complex_=False):
    sects, sizes = st.allsectorsandsizes(charge, space)
    blocks = {}
    for s, z in zip(sects, sizes):
        b = rng.random(z)
        if complex_:
            b = b + 1j * rng.random(z)
        blocks[s] = b
    return st.SymTensor(charge, space, blocks)


def test_fuse_split_exact():
    """symtensortests.jl:3-29 "fuse/split"."""
    space = (U1Space((0, 2), (1, 3)), U1Space((0, 1), (1, 1)), dual(U1Space((0, 3), (1, 4))))
    sects = [(0, 0, 0), (0, 1, 1), (1, 0, 1)]
    blks = [np.arange(1, 7).reshape((2, 1, 3), order="F"),
            np.arange(7, 15).reshape((2, 1, 4), order="F"),
            np.arange(15, 27).reshape((3, 1, 4), order="F")]
    A0 = st.SymTensor(0, space, dict(zip(sects, blks)))
    A1 = st.fuselegs(A0, 1, 2)
    assert st.splitleg(A1, 1, space[0:2]) == A0
    A1 = st.fuselegs(A0, 2, 2, True)
    assert st.splitleg(A1, 2, space[1:3]) == A0


def test_u1_unitary_sector_order_and_values():
    """symtensortests.jl:41-53 "U1 unitary": pins the sector order after two splits."""
    A = st.eye(U1Space((0, 1), (1, 2), (2, 1)))
    A[(1, 1)] = np.array([[2.0, 3.0], [4.0, 5.0]])
    d = U1Space((0, 1), (1, 1))
    B = st.splitleg(st.splitleg(A, 2, (dual(d), dual(d))), 1, (d, d))
    expected = sorted([(1, 1, 1, 1), (1, 0, 0, 1), (0, 1, 0, 1), (1, 0, 1, 0), (0, 1, 1, 0),
                       (0, 0, 0, 0)], key=st.sector_key)
    assert B.sectors() == expected
    i = np.ones((1, 1, 1, 1))
    vals = list(B.blocks.values())
    for got, want in zip(vals, [i, 2 * i, 4 * i, 3 * i, 5 * i, 1 * i]):
        assert np.array_equal(got, want)


def test_symmatrix_layout_matches_fuselegs():
    """symtensortests.jl:76-92 "converts" (every permutation instead of one random one)."""
    vlist = (U1Space((0, 2), (1, 3), (2, 4)), U1Space((-2, 4), (-1, 3), (0, 2), (1, 1)),
             U1Space((-1, 1), (0, 2), (1, 3), (2, 4)), U1Space((-2, 3), (-1, 2), (0, 1)))
    A = st.fill_linearindex(0, vlist)
    M = st.symmatrix(A, [1, 2], [3, 4])
    assert M == st.fuselegs(st.fuselegs(A, 3, 2, True), 1, 2)
    assert M == st.fuselegs(st.fuselegs(A, 1, 2), 2, 2, True)
    for perm in itertools.permutations([1, 2, 3, 4]):
        perm = list(perm)
        assert st.symmatrix(A, perm[:2], perm[2:]) == st.fuselegs(
            st.fuselegs(st.permutelegs(A, perm), 3, 2, True), 1, 2)


def test_contract_matrices_exact():
    """symtensortests.jl:94-110 "matrices": exact equality with the dense product."""
    vlist = (U1Space((0, 2), (1, 3), (2, 4)), dual(U1Space((0, 4), (1, 2), (2, 2), (3, 3))),
             U1Space((0, 4), (1, 2), (2, 2), (3, 3)), dual(U1Space((0, 3), (1, 5), (2, 2))))
    A = st.fill_linearindex(0, vlist[0:2])
    B = st.fill(1.0, 0, vlist[2:4])
    C = st.contract(A, (1, -1), B, (-1, 2))
    assert np.array_equal(st.array(A) @ st.array(B), st.array(C))


def test_contract_multi_leg_vs_dense():
    """symtensortests.jl:112-137 "multi leg tensors"."""
    rng = np.random.default_rng(1911)
    vlist = (U1Space((0, 2), (1, 2), (2, 2)), U1Space((0, 2), (-1, 2), (-2, 2), (-3, 2)),
             U1Space((0, 2), (1, 2), (2, 2)), dual(U1Space((0, 2), (1, 2))),
             U1Space((0, 2), (1, 2)), U1Space((0, 2), (1, 2), (2, 2), (3, 2), (4, 2)),
             U1Space((0, 2), (1, 2)), U1Space((0, 2), (-1, 2), (-2, 2)))
    A = rand_tensor(0, vlist[0:4], rng)
    B = rand_tensor(0, vlist[4:8], rng)
    assert st.splitleg(st.fuselegs(A, 1, 3), 1, vlist[0:3]).isapprox(A)
    assert st.splitleg(st.fuselegs(A, 2, 2), 2, vlist[1:3]).isapprox(A)
    assert st.splitleg(st.fuselegs(A, 2, 3), 2, vlist[1:4]).isapprox(A)
    C = st.contract(A, (1, 2, 3, -1), B, (-1, 4, 5, 6))
    C_ = np.einsum("abcd,defg->abcefg", st.array(A), st.array(B))
    np.testing.assert_allclose(st.array(C), C_, rtol=1e-12, atol=1e-12)


def test_dot_complex_vs_dense():
    """symtensortests.jl:151-155 "dot"."""
    rng = np.random.default_rng(7)
    vlist = (U1Space((0, 2), (1, 3), (2, 4)), U1Space((0, 4), (-1, 2), (-2, 2), (-3, 3)),
             U1Space((0, 3), (1, 5), (2, 2)), U1Space((0, 6), (-1, 7)))
    A = rand_tensor(0, vlist, rng, complex_=True)
    A_ = st.array(A)
    assert np.isclose(np.vdot(A_, A_), st.dot(A, A))


@pytest.mark.parametrize("charge", [0, 1, -1])
@pytest.mark.parametrize("cplx", [False, True])
def test_svd_reconstruction(charge, cplx):
    """symtensortests.jl:165-185 "svd": u*s*v ≈ A for charges 0, ±1, real and complex."""
    rng = np.random.default_rng(11 + charge)
    V1 = U1Space((0, 2), (1, 3), (2, 4))
    V2 = U1Space((0, 4), (-1, 2), (-2, 2), (-3, 3))
    V3 = U1Space((0, 4), (1, 2), (2, 2), (3, 3))
    space = (V1, dual(V3)) if cplx else (V1, V2)
    A = rand_tensor(charge, space, rng, complex_=cplx)
    u, s, v = st.svd_(A)
    assert st.matmul(st.matmul(u, s), v).isapprox(A, rtol=1e-10)


def test_svdtrunc_equals_svd_without_truncation():
    """symtensortests.jl:187-190 "svdtrunc"."""
    rng = np.random.default_rng(3)
    A = rand_tensor(0, (U1Space((0, 2), (1, 3), (2, 4)), U1Space((0, 4), (-1, 2), (-2, 2), (-3, 3))),
                    rng, complex_=True)
    u0, s0, v0 = st.svd_(A)
    u1, s1, v1 = st.svdtrunc(A)
    assert u0.isapprox(u1) and v0.isapprox(v1)
    assert all(np.allclose(s0.blocks[k], s1.blocks[k]) for k in s0.blocks)


def test_xxz_u1mpo_blocks_equal_ed_blocks():
    """mpotests.jl:3-58 "xxz": the U(1) MPO of 4 sites equals the ED Hamiltonian in every
    particle-number block, exactly."""
    Ws = om.xxz_u1mpo(4, 1.0)
    c = st.contract
    h4 = c(c(c(Ws[0], (1, 2, -1, 5), Ws[1], (-1, 3, 4, 6)), (1, 2, 3, -1, 6, 7),
             Ws[2], (-1, 4, 5, 8)), (1, 2, 3, 4, -1, 7, 8, 9), Ws[3], (-1, 5, 6, 10))
    h4 = st.fuselegs(st.fuselegs(h4, 1, 5), 2, 5, True)
    H4 = om.xxz_hamiltonian(4, 1.0)
    pop = np.array([bin(n).count("1") for n in range(16)])
    for k in range(5):
        idx = np.where(pop == k)[0]
        assert np.array_equal(H4[np.ix_(idx, idx)], h4.blocks[(k, k)])


@pytest.mark.parametrize("lx", [2, 3, 4, 5])
def test_xxz_hamiltonian_small(lx):
    """mpotests.jl:42-44 compares the dense MPO with ``xxz_hamiltonian``; here the U(1) MPO,
    fully contracted and embedded densely, is compared with the same Hamiltonian."""
    Ws = om.xxz_u1mpo(lx, 0.7)
    h = Ws[0]
    for k in range(1, lx):
        idxh = (1,) + tuple(range(2, k + 2)) + (-1,) + tuple(range(k + 4, 2 * k + 4))
        idxw = (-1, k + 2, k + 3, 2 * k + 4)
        h = st.contract(h, idxh, Ws[k], idxw)
    # legs: V0, s_1..s_L, Vend, s'_1..s'_L; the bond legs have dimension 1
    dense = st.array(h).reshape((2,) * (2 * lx), order="F")
    # charge 0 (spin down) is dense basis index 2 of the reference, and site 1 is the slowest
    # index of its Kronecker products
    dense = np.flip(dense, axis=tuple(range(2 * lx)))
    mat = dense.reshape((2 ** lx, 2 ** lx), order="C")
    np.testing.assert_allclose(mat, om.xxz_hamiltonian(lx, 0.7), atol=1e-14)


def test_dmrg_energy_matches_exact_diagonalisation():
    """Restates the intent of mpstests.jl:24-31 (MPS energy == ED energy) for the symmetric
    2-site DMRG path: L=10 Heisenberg chain, Sz=0, exact ground energy from the dense
    Hamiltonian restricted to half filling."""
    lx, M = 10, 5
    rng = np.random.default_rng(1911)
    Ws = om.xxz_u1mpo(lx, 1.0)
    mps = random_mps(lx, M, 16, rng)
    om.center_at(mps, 1)
    env = om.initialenv(mps, Ws)
    for _ in range(3):
        es = om.dmrg2sitesweep(mps, Ws, env, maxdim=32, tol=1e-12, krylovdim=4, krylovmaxiter=20,
                               lanczostol=1e-10)
    H = om.xxz_hamiltonian(lx, 1.0)
    pop = np.array([bin(n).count("1") for n in range(2 ** lx)])
    idx = np.where(pop == M)[0]
    e0 = np.linalg.eigvalsh(H[np.ix_(idx, idx)])[0]
    assert len(es) == 3 * lx - 5
    assert abs(es[-1] - e0) < 1e-9


def random_mps(lx, M, chimax, rng):
    d = U1Space((0, 1), (1, 1))
    Vl = U1Space((0, 1))
    As = []
    for site in range(1, lx + 1):
        Vr = U1Space(*om.binomial_bond_dims(lx, site, M, chimax))
        As.append(rand_tensor(0, (Vl, d, dual(Vr)), rng))
        Vl = Vr
    return om.MPState(As, 0)


@pytest.mark.parametrize("bond", [1, 3, 6])
def test_lanczos_restatement_finds_the_lowest_eigenpair_of_heff(bond):
    """The KrylovKit boundary is unpinned against Julia; its restatement (thick-restart Lanczos,
    krylovdim 5 as in dmrg.jl:63-65) is checked against the dense spectrum of the same two-site
    operator (apply.jl:93-105) at an inner bond of an L=8 Heisenberg chain: lowest eigenvalue
    to 1e-10 and a normalised eigenvector with residual below the tolerance."""
    from mps_gb300 import dmrg as gd
    lx, chi = 8, 8
    sites = gd.random_mps_host(lx, lx // 2, chi, seed=11)
    conv = lambda sp: tuple(st.VectorSpace(V.sectors, V.isdual) for V in sp)
    mps = om.MPState([st.from_flat(c, conv(sp), f) for c, sp, f in sites], 0)
    om.center_at(mps, bond)
    Ws = om.xxz_u1mpo(lx, 1.0)
    env = om.initialenv(mps, Ws, at=bond)
    v0 = st.contract(mps.As[bond - 1], (1, 2, -1), mps.As[bond], (-1, 3, 4))
    f = om._heff(env, Ws, bond)
    flat0 = st.flatten(v0)
    n = flat0.size
    H = np.zeros((n, n))
    for i in range(n):
        e = np.zeros(n)
        e[i] = 1.0
        H[:, i] = st.flatten(f(st.from_flat(v0.charge, v0.space, e)))
    np.testing.assert_allclose(H, H.T, atol=1e-12)
    w = np.linalg.eigvalsh(H)
    theta, x, info = om.eigsolve_lanczos(f, v0, krylovdim=5, maxiter=200, tol=1e-11)
    assert info.converged
    assert abs(theta - w[0]) < 1e-10 * max(1.0, abs(w[0]))
    xf = st.flatten(x)
    assert abs(np.linalg.norm(xf) - 1.0) < 1e-12
    assert np.linalg.norm(H @ xf - theta * xf) < 1e-9
