"""Lattice MPOs (the role of src/mpogen.jl:153-352): the finite-state-machine U(1) MPO, contracted
to a dense matrix on the host, equals the Hamiltonian assembled directly from its terms by
Kronecker products; bond dimensions count the open terms."""
import numpy as np
import pytest

from mps_gb300 import lattice as lt


def dense_from_terms(n, terms):
    """Sum over terms of kron(op at each site, identity elsewhere); site 0 most significant,
    basis (down, up)."""
    H = np.zeros((2 ** n, 2 ** n))
    for sites, ops, amp in terms:
        mats = [np.eye(2)] * n
        mats = list(mats)
        for s, o in zip(sites, ops):
            mats[s] = lt.OPS[o][0]
        M = mats[0]
        for m in mats[1:]:
            M = np.kron(M, m)
        H += amp * M
    return H


def test_chain_mpo_equals_dense_xxz():
    n = 6
    terms = lt.chain_xxz_terms(n, 0.7)
    H = lt.dense_mpo(lt.mpo_blocks(n, terms))
    np.testing.assert_allclose(H, dense_from_terms(n, terms), atol=1e-14)
    # the XXZ chain needs 2 + 3 channels on every inner bond (the reference's w = 5)
    for (Vl, _, Vr, _), _ in lt.mpo_blocks(n, terms)[1:-1]:
        assert sum(Vl[1]) == 5


@pytest.mark.parametrize("width,length", [(3, 2), (4, 2), (2, 3)])
def test_cylinder_mpo_equals_dense(width, length):
    n = width * length
    terms = lt.cylinder_heisenberg_terms(width, length)
    H = lt.dense_mpo(lt.mpo_blocks(n, terms))
    np.testing.assert_allclose(H, dense_from_terms(n, terms), atol=1e-13)
    # Heisenberg: H commutes with the total Sz (U(1)) and is symmetric
    np.testing.assert_allclose(H, H.T, atol=1e-14)


def test_cylinder_bond_dimension():
    """6 x 24 cylinder: a cut at a column boundary crosses the 6 bonds along the length
    (3 terms each, w = 2 + 18 = 20); a cut inside a column also crosses one bond around the
    circumference and the wrap bond (w = 26)."""
    width, length = 6, 24
    terms = lt.cylinder_heisenberg_terms(width, length)
    tens = lt.mpo_blocks(width * length, terms)
    dims = [sum(Vr[1]) for (_, _, Vr, _), _ in tens]
    assert dims[width - 1] == 20 and dims[2 * width - 1] == 20
    assert max(dims) == 2 + 3 * (width + 2)
    assert dims[-1] == 1


def test_bad_terms_rejected():
    with pytest.raises(ValueError):
        lt.mpo_blocks(4, [((2, 1), ("P", "M"), 1.0)])
    with pytest.raises(ValueError):
        lt.mpo_blocks(3, [((1, 3), ("Z", "Z"), 1.0)])


# ---- j1j2 chain and triangular lattice (src/spinmodels.jl:14-110; test/mpotests.jl:108-185) ----
def _perm_dense(n, cycle):
    """P + P^T for the permutation that moves the spin at cycle[k] to cycle[k+1] (site 0 the
    most significant bit): a swap for two sites, the ring exchange for four."""
    P = np.zeros((2 ** n, 2 ** n))
    for j in range(2 ** n):
        bits = [(j >> (n - 1 - s)) & 1 for s in range(n)]
        new = list(bits)
        for k, s in enumerate(cycle):
            new[cycle[(k + 1) % len(cycle)]] = bits[s]
        i = sum(b << (n - 1 - s) for s, b in enumerate(new))
        P[i, j] += 1.0
    return P + P.T


def _heis_dense(n, bonds):
    """sum J S_i.S_j with S_i.S_j = swap/2 - 1/4 (swap = (P + P^T)/2 for two sites)."""
    H = np.zeros((2 ** n, 2 ** n))
    for i, j, J in bonds:
        H += J * (0.25 * _perm_dense(n, [i, j]) - 0.25 * np.eye(2 ** n))
    return H


def _j1j2_dense(n, j1, j2):
    return _heis_dense(n, [(i, i + 1, j1) for i in range(n - 1)] +
                       [(i, i + 2, j2) for i in range(n - 2)])


def _popcount_blocks_only(H, n):
    pc = np.array([bin(i).count("1") for i in range(2 ** n)])
    return np.all(H[pc[:, None] != pc[None, :]] == 0)


@pytest.mark.parametrize("lx", [3, 4, 6])
def test_j1j2_chain_mpo_equals_explicit(lx):
    j1, j2 = 1.0, 0.3
    H = lt.dense_mpo(lt.mpo_blocks(lx, lt.j1j2_chain_terms(lx, j1, j2)))
    np.testing.assert_allclose(H, _j1j2_dense(lx, j1, j2), atol=1e-14)
    assert _popcount_blocks_only(H, lx)


@pytest.mark.parametrize("n", [2, 3])
def test_two_leg_triangular_ladder_is_the_j1j2_chain(n):
    """mpotests.jl:126-137: the (2, n) triangular ladder with couplings (0.3, 1, 1) is the
    zigzag j1j2 chain of 2n sites (j1 = 1, j2 = 0.3)."""
    H = lt.dense_mpo(lt.mpo_blocks(2 * n, lt.triangular_terms(2, n, 0.3, 1.0, 1.0)))
    np.testing.assert_allclose(H, _j1j2_dense(2 * n, 1.0, 0.3), atol=1e-14)


def test_two_leg_triangle_with_ring_exchange():
    """mpotests.jl:140-162: the (2, 4) ladder with ring exchanges k1, k2 equals the j1j2 chain
    plus the four-spin ring (cyclic order 1, 3, 4, 2 of each window of four consecutive sites;
    k1 on windows starting at even sites, k2 at odd), up to the constant that R4 - 1/4 removes."""
    n, j1, j2, k1, k2 = 4, 1.0, 0.3, 0.4, 0.7
    L = 2 * n
    H = _j1j2_dense(L, j1, j2)
    nk = {k1: 0, k2: 0}
    for w in range(L - 3):
        k = k1 if w % 2 == 0 else k2
        H += k * _perm_dense(L, [w, w + 2, w + 3, w + 1])
        nk[k] += 1
    terms = lt.triangular_terms(2, n, j2, j1, j1, k1, k2, 0.0)
    Hmpo = lt.dense_mpo(lt.mpo_blocks(L, terms))
    shift = 0.25 * (k1 * nk[k1] + k2 * nk[k2])
    np.testing.assert_allclose(Hmpo + shift * np.eye(2 ** L), H, atol=1e-12)
    assert _popcount_blocks_only(Hmpo, L)


@pytest.mark.parametrize("ly,lx,periodic", [(2, 2, False), (2, 3, False), (3, 2, True)])
def test_triangular_mpo_with_random_couplings(ly, lx, periodic):
    """mpotests.jl:165-185: random j1..k3; the U(1) MPO is the Hamiltonian assembled from
    swaps and ring permutations on the same bonds and plaquettes."""
    rng = np.random.default_rng(ly * 10 + lx)
    j1, j2, j3, k1, k2, k3 = rng.random(6)
    n = ly * lx
    Hmpo = lt.dense_mpo(lt.mpo_blocks(n, lt.triangular_terms(ly, lx, j1, j2, j3, k1, k2, k3,
                                                             periodic_y=periodic)))
    site = lambda y, x: (x * ly + (y % ly if periodic else y)
                         if (periodic or 0 <= y < ly) and 0 <= x < lx else None)
    H = np.zeros((2 ** n, 2 ** n))
    for x in range(lx):
        for y in range(ly):
            for J, (dy, dx) in ((j1, (0, 1)), (j2, (1, 0)), (j3, (1, -1))):
                t = site(y + dy, x + dx)
                if t is not None:
                    H += _heis_dense(n, [(site(y, x), t, J)])
            for K, offs in ((k1, ((0, 0), (0, 1), (1, 1), (1, 0))),
                            (k2, ((0, 0), (0, 1), (1, 0), (1, -1))),
                            (k3, ((0, 0), (1, 0), (0, 1), (-1, 1)))):
                ss = [site(y + dy, x + dx) for dy, dx in offs]
                if None not in ss:
                    H += K * (_perm_dense(n, ss) - 0.25 * np.eye(2 ** n))
    np.testing.assert_allclose(Hmpo, H, atol=1e-12)
    np.testing.assert_allclose(Hmpo, Hmpo.T, atol=1e-13)
    assert _popcount_blocks_only(Hmpo, n)


def test_ring_expansion_reassembles_the_ring_operator():
    terms = lt.ring_exchange_terms([0, 1, 2, 3], 1.0)
    H = lt.dense_mpo(lt.mpo_blocks(4, terms))
    np.testing.assert_allclose(H, _perm_dense(4, [0, 1, 2, 3]) - 0.25 * np.eye(16), atol=1e-14)


# ---- channels shared by open terms with the same placed operators ----
def _max_bond(blocks):
    return max(sum(Vl[1]) for (Vl, _, _, _), _ in blocks)


@pytest.mark.parametrize("n,make", [
    (8, lambda: lt.chain_xxz_terms(8, 0.7)),
    (9, lambda: lt.j1j2_chain_terms(9, 1.0, 0.3)),
    (8, lambda: lt.triangular_terms(2, 4, 0.3, 1.0, 1.0, 0.4, 0.7)),
    (6, lambda: lt.triangular_terms(3, 2, 0.2, 0.3, 0.4, 0.5, 0.6, 0.7, periodic_y=True)),
    (9, lambda: lt.cylinder_heisenberg_terms(3, 3)),
])
def test_shared_prefix_mpo_is_the_same_hamiltonian(n, make):
    terms = make()
    full = lt.mpo_blocks(n, terms)
    shared = lt.mpo_blocks(n, terms, share_prefixes=True)
    np.testing.assert_allclose(lt.dense_mpo(shared), lt.dense_mpo(full), atol=1e-12)
    np.testing.assert_allclose(lt.dense_mpo(shared), dense_from_terms(n, terms), atol=1e-12)
    assert _max_bond(shared) <= _max_bond(full)


def test_shared_prefixes_shrink_the_bond_dimension():
    """The 6 x 24 cylinder reaches w = 2 + 3 W = 20 at every cut (26 with one channel per
    term); the j1j2 chain 8 (11); the ring-exchange ladder 33 (86)."""
    cases = [(144, lt.cylinder_heisenberg_terms(6, 24), 26, 20),
             (64, lt.j1j2_chain_terms(64, 1.0, 0.3), 11, 8),
             (64, lt.triangular_terms(2, 32, 0.3, 1.0, 1.0, 0.4, 0.7), 86, 33)]
    for n, terms, w_full, w_shared in cases:
        assert _max_bond(lt.mpo_blocks(n, terms)) == w_full
        assert _max_bond(lt.mpo_blocks(n, terms, share_prefixes=True)) == w_shared


def test_duplicate_terms_add_on_the_shared_finishing_edge():
    terms = [((0, 2), ("Z", "Z"), 0.25), ((0, 2), ("Z", "Z"), 0.5), ((1,), ("Z",), 1.0),
             ((1,), ("Z",), -0.5)]
    shared = lt.mpo_blocks(3, terms, share_prefixes=True)
    np.testing.assert_allclose(lt.dense_mpo(shared), dense_from_terms(3, terms), atol=1e-15)
    assert _max_bond(shared) == 3  # done, the one shared Z channel, start


def test_structure_only_device_mpo_with_shared_prefixes():
    Ws = lt.device_mpo(144, lt.cylinder_heisenberg_terms(6, 24), meta_only=True,
                       share_prefixes=True)
    assert max(W.space[0].dim() for W in Ws) == 20
    assert Ws[0].space[0].dim() == 1 and Ws[-1].space[2].dim() == 1
